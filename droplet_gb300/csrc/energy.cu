// energy.cu -- in-situ turbulence and free-energy diagnostics of the current
// fields (dl_energy):
//  * the shell-binned kinetic-energy spectrum of enesupe_cal,
//    program/turbulence_hit_xy.f90:588-645: u_hat = FFT(u)/N (fft_r2c,
//    :725-730), summed over the reference's index set k1 in [0,nx),
//    k2 in [0,ny), k3 in [0,nz/2] with weight 1 on k3 = 0 and 2 elsewhere,
//    into bin int(|k|) + 1 with the signed wavenumbers of the function judge (:739-746);
//    the FFTs are cuFFT D2Z transforms in FP64, modes outside the stored half
//    are read through Hermitian symmetry;
//  * sums of the bulk free energy psi = phi T ln(phi/(1 - b phi)) - a phi^2
//    (free_energy_cal, program/energy_budget.f90:1012-1023), of the chemical
//    potential mu = T ln(phi/(1 - b phi)) + T/(1 - b phi) - 2 a phi
//    - kappag lap(phi) (chemical_potencial_cal, :998-1010; the 14-neighbour
//    Laplacian of various_cal) and of |grad phi|^2.
#include "dl_internal.cuh"

#include <cufft.h>
#include <math.h>
#include <string.h>
#include <vector>

namespace dl {

constexpr int EN_THREADS = 256;
constexpr int EN_BLOCKS = 304;
constexpr int EN_SMEM_BINS = 2048;  // bins histogrammed in shared memory first

// one velocity component as doubles (the FFT input)
__global__ void en_component(const void* mac, int fast, int c, long long N, double* __restrict__ out) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= N) return;
    out[s] = fast ? (double)((const float*)mac)[(c + 1) * N + s] : ((const double*)mac)[(c + 1) * N + s];
}

// acc += |u_hat|^2 / N^2 over the stored half spectrum
__global__ void en_accumulate(const cufftDoubleComplex* __restrict__ uh, long long M, double invN2, int first,
                              double* __restrict__ acc) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M) return;
    const double v = (uh[t].x * uh[t].x + uh[t].y * uh[t].y) * invN2;
    acc[t] = first ? v : acc[t] + v;
}

__device__ __forceinline__ int en_signed(int k, int n) { return k >= n / 2 + 1 ? k - n : k; }

// spectrum[int(|k|)] += 0.5 |u_hat|^2 w over the reference's index set
__global__ void __launch_bounds__(EN_THREADS) en_bin(const double* __restrict__ acc, int nx, int ny, int nz,
                                                    int nbins, double* __restrict__ spectrum) {
    __shared__ double hist[EN_SMEM_BINS];
    const int nsh = nbins < EN_SMEM_BINS ? nbins : EN_SMEM_BINS;
    for (int b = threadIdx.x; b < nsh; b += blockDim.x) hist[b] = 0.0;
    __syncthreads();
    const int nxh = nx / 2 + 1;
    const long long total = (long long)nx * ny * (nz / 2 + 1);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k1 = (int)(t % nx);
        const long long r = t / nx;
        const int k2 = (int)(r % ny);
        const int k3 = (int)(r / ny);
        // stored index [iz][iy][ix] of (k1, k2, k3) or of its partner -k
        int ix = k1, iy = k2, iz = k3;
        if (k1 >= nxh) {
            ix = nx - k1;
            iy = (ny - k2) % ny;
            iz = (nz - k3) % nz;
        }
        const double e2 = acc[((long long)iz * ny + iy) * nxh + ix];
        const int s1 = en_signed(k1, nx), s2 = en_signed(k2, ny), s3 = en_signed(k3, nz);
        const int kidx = (int)sqrt((double)(s1 * s1 + s2 * s2 + s3 * s3));  // bin index - 1
        if (kidx >= nbins) continue;
        const double v = 0.5 * e2 * (k3 == 0 ? 1.0 : 2.0);
        if (kidx < nsh) atomicAdd(hist + kidx, v);
        else atomicAdd(spectrum + kidx, v);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nsh; b += blockDim.x)
        if (hist[b] != 0.0) atomicAdd(spectrum + b, hist[b]);
}

// per-block partial sums of psi, mu and |grad phi|^2
struct EnArgs {
    int nx, ny, nz;
    long long N;
    const void* mac;
    int fast;
    double phi_off, T, a, b, kappag, inv_lap, inv_grad;
    double* part;  // [EN_BLOCKS][3]
};

__device__ __forceinline__ double en_phi(const EnArgs& a, long long s) {
    return a.fast ? a.phi_off + (double)((const float*)a.mac)[s] : ((const double*)a.mac)[s];
}

__device__ __forceinline__ long long en_wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

__global__ void __launch_bounds__(EN_THREADS) en_free_energy(const EnArgs a) {
    double acc[3] = {0.0, 0.0, 0.0};
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < a.N;
         s += (long long)gridDim.x * blockDim.x) {
        const long long row = s / a.nx;
        const int x = (int)(s - row * a.nx);
        const int z = (int)(row / a.ny);
        const int y = (int)(row - (long long)z * a.ny);
        const double ph = en_phi(a, s);
        double lap = -(14.0 * ph), g[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int i = 1; i < Q; ++i) {
            const long long nb = en_wrap(x + cx(i), a.nx) +
                                 (long long)a.nx * (en_wrap(y + cy(i), a.ny) + (long long)a.ny * en_wrap(z + cz(i), a.nz));
            const double v = en_phi(a, nb);
            lap = lap + v;
            g[0] += cx(i) * v;
            g[1] += cy(i) * v;
            g[2] += cz(i) * v;
        }
        lap = lap * a.inv_lap;
        const double omb = 1.0 - a.b * ph;
        const double lg = log(ph / omb);
        acc[0] += ph * a.T * lg - a.a * ph * ph;
        acc[1] += (a.T * lg + a.T / omb - 2.0 * a.a * ph) - a.kappag * lap;
        acc[2] += (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) * a.inv_grad * a.inv_grad;
    }
    __shared__ double sh[EN_THREADS / 32][3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
        for (int w = 0; w < EN_THREADS / 32; ++w) v += sh[w][threadIdx.x];
        a.part[blockIdx.x * 3 + threadIdx.x] = v;
    }
}

void energy_free(dl_handle* h) {
    if (h->en_plan_ok) cufftDestroy((cufftHandle)h->en_plan);
    h->en_plan_ok = 0;
    cudaFree(h->en_buf);
    h->en_buf = nullptr;
}

static int en_spectrum(dl_handle* h, double* spectrum_host, long long nbins, double* spec_sum) {
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const long long N = (long long)h->N;
    const long long M = (long long)nz * ny * (nx / 2 + 1);  // stored half spectrum
    // buffer: input N doubles | output M complex | acc M doubles | bins
    double* in = h->en_buf;
    cufftDoubleComplex* out = (cufftDoubleComplex*)(in + N + (N & 1));
    double* acc = (double*)(out + M);
    double* bins = acc + M;
    if (!h->en_plan_ok) {
        cufftHandle plan;
        if (cufftPlan3d(&plan, nz, ny, nx, CUFFT_D2Z) != CUFFT_SUCCESS)
            return set_error(h, DL_ERR_CUDA, "cufftPlan3d(D2Z) failed");
        h->en_plan = (long long)plan;
        h->en_plan_ok = 1;
    }
    const cufftHandle plan = (cufftHandle)h->en_plan;
    if (cufftSetStream(plan, h->stream) != CUFFT_SUCCESS) return set_error(h, DL_ERR_CUDA, "cufftSetStream failed");
    const bool fast = h->form != DL_FORM_FP64;
    const void* mac = fast ? (const void*)h->mac32[h->cur] : (const void*)h->mac64[h->cur];
    const double invN2 = 1.0 / ((double)N * (double)N);
    for (int c = 0; c < 3; ++c) {
        DL_LAUNCH(h, false, (en_component<<<(unsigned)((N + 255) / 256), 256, 0, h->stream>>>(mac, fast, c, N, in)));
        if (cufftExecD2Z(plan, in, out) != CUFFT_SUCCESS) return set_error(h, DL_ERR_CUDA, "cufftExecD2Z failed");
        DL_LAUNCH(h, false,
                  (en_accumulate<<<(unsigned)((M + 255) / 256), 256, 0, h->stream>>>(out, M, invN2, c == 0, acc)));
    }
    DL_CUDA(h, cudaMemsetAsync(bins, 0, sizeof(double) * (size_t)nbins, h->stream));
    DL_LAUNCH(h, false, (en_bin<<<EN_BLOCKS, EN_THREADS, 0, h->stream>>>(acc, nx, ny, nz, (int)nbins, bins)));
    DL_CUDA(h, cudaGetLastError());
    DL_CUDA(h, cudaMemcpyAsync(spectrum_host, bins, sizeof(double) * (size_t)nbins, cudaMemcpyDeviceToHost,
                               h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    double s = 0.0;
    for (long long b = 0; b < nbins; ++b) s += spectrum_host[b];
    *spec_sum = s;
    return DL_OK;
}

int energy_diagnostics(dl_handle* h, dl_energy_diag* out, double* spectrum_host, long long nbins) {
    if (nbins < 0 || (nbins > 0 && !spectrum_host)) return set_error(h, DL_ERR_ARG, "bad spectrum buffer");
    const long long N = (long long)h->N;
    const long long M = (long long)h->nz * h->ny * (h->nx / 2 + 1);
    const size_t need = sizeof(double) * (size_t)(N + 1 + 2 * M + M + (nbins > 0 ? nbins : 0) + 3 * EN_BLOCKS);
    if (need > h->en_bytes) {
        cudaFree(h->en_buf);
        h->en_buf = nullptr;
        h->en_bytes = 0;
        DL_CUDA(h, cudaMalloc(&h->en_buf, need));
        h->en_bytes = need;
    }
    memset(out, 0, sizeof(*out));
    // free-energy sums (partials at the end of the buffer)
    EnArgs a;
    memset(&a, 0, sizeof(a));
    a.nx = h->nx;
    a.ny = h->ny;
    a.nz = h->nz;
    a.N = N;
    a.fast = h->form != DL_FORM_FP64;
    a.mac = a.fast ? (const void*)h->mac32[h->cur] : (const void*)h->mac64[h->cur];
    a.phi_off = h->P.phi1;
    a.T = h->P.T;
    a.a = h->P.a;
    a.b = h->P.b;
    a.kappag = h->P.kappag;
    a.inv_lap = 1.0 / (5.0 * h->P.ds * h->P.ds);
    a.inv_grad = 1.0 / (10.0 * h->P.ds);
    a.part = h->en_buf + h->en_bytes / sizeof(double) - 3 * EN_BLOCKS;
    DL_LAUNCH(h, false, (en_free_energy<<<EN_BLOCKS, EN_THREADS, 0, h->stream>>>(a)));
    DL_CUDA(h, cudaGetLastError());
    std::vector<double> part(3 * EN_BLOCKS);
    DL_CUDA(h, cudaMemcpyAsync(part.data(), a.part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    double sums[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < EN_BLOCKS; ++b)
        for (int k = 0; k < 3; ++k) sums[k] += part[3 * b + k];
    out->psi_sum = sums[0];
    out->mu_sum = sums[1];
    out->grad_sq_sum = sums[2];
    out->nbins = nbins;
    if (nbins > 0) {
        int rc = en_spectrum(h, spectrum_host, nbins, &out->spectrum_sum);
        if (rc != DL_OK) return rc;
    }
    out->step = h->step;
    return DL_OK;
}

}  // namespace dl
