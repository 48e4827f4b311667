// reduce.cu -- FP64 whole-domain diagnostics of the macroscopic fields (the
// per-site terms of diag_site.cuh: conservation sums, kinetic energy,
// dissipation, droplet volume, pressure inside/outside, deformation moments).
//
// Two launches: per-block partial sums (one pass over the fields, per-thread
// FP64 accumulators, warp-shuffle then shared-memory tree), then one warp
// that adds the partials of every block in a fixed order with Neumaier
// compensation, so the result is deterministic.
#include "dl_internal.cuh"
#include "diag_site.cuh"

#include <string.h>

namespace dl {

constexpr int NSUM = DIAG_NSUM;  // sums, then min, max
constexpr int NPART = NSUM + 2;
constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs
constexpr int RED_THREADS = 256;

struct RedArgs {
    DiagConsts k;
    double* part;
};

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) reduce_partials(const T* __restrict__ mac, const RedArgs a) {
    double acc[NSUM];
#pragma unroll
    for (int k = 0; k < NSUM; ++k) acc[k] = 0.0;
    double vmin = INFINITY, vmax = -INFINITY;
    diag_sites(mac, a.k, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, acc, vmin,
               vmax);
    __shared__ double sh[RED_THREADS / 32][NPART];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NSUM; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][k] = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vmin = fmin(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    if (lane == 0) {
        sh[warp][NSUM] = vmin;
        sh[warp][NSUM + 1] = vmax;
    }
    __syncthreads();
    if (threadIdx.x < NPART) {
        const int k = threadIdx.x;
        double v = sh[0][k];
        for (int w = 1; w < RED_THREADS / 32; ++w) {
            if (k == NSUM) v = fmin(v, sh[w][k]);
            else if (k == NSUM + 1) v = fmax(v, sh[w][k]);
            else v += sh[w][k];
        }
        a.part[(long long)blockIdx.x * NPART + k] = v;
    }
}

__global__ void reduce_final(const double* __restrict__ part, int nblocks, double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k >= NPART) return;
    if (k == NSUM || k == NSUM + 1) {
        double v = part[k];
        for (int b = 1; b < nblocks; ++b) v = (k == NSUM) ? fmin(v, part[b * NPART + k]) : fmax(v, part[b * NPART + k]);
        out[k] = v;
        return;
    }
    // Neumaier-compensated sum in block order
    double s = 0.0, c = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        const double v = part[b * NPART + k];
        const double t = s + v;
        if (fabs(s) >= fabs(v)) c += (s - t) + v;
        else c += (v - t) + s;
        s = t;
    }
    out[k] = s + c;
}

// the per-site constants of the diagnostics for handle h (shared with dl_reduce_static)
void diag_consts(const dl_handle* h, double phi_off, double p_off, DiagConsts& k) {
    k.nx = h->nx;
    k.ny = h->ny;
    k.nz = h->nz;
    k.N = (long long)h->N;
    k.phi1 = h->P.phi1;
    k.phi_off = phi_off;
    k.p_off = p_off;
    k.inv_span = 1.0 / (h->P.phi2 - h->P.phi1);
    k.mid = 0.5 * (h->P.phi1 + h->P.phi2);
    k.nu1 = h->P.nu1;
    k.dnu = h->P.nu2 - h->P.nu1;
    const double graddiv = 10.0 * h->P.ds;
    k.sfac = 1.0 / (4.0 * graddiv * graddiv);
}

template <typename T>
static int reduce_any(dl_handle* h, const T* d_mac, double phi_off, double p_off, dl_diag* out) {
    if (!h->d_diag) DL_CUDA(h, cudaMalloc(&h->d_diag, sizeof(double) * (RED_BLOCKS * NPART + NPART)));
    RedArgs a;
    memset(&a, 0, sizeof(a));
    diag_consts(h, phi_off, p_off, a.k);
    a.part = h->d_diag;
    DL_LAUNCH(h, false, reduce_partials<T><<<RED_BLOCKS, RED_THREADS, 0, h->stream>>>(d_mac, a));
    DL_LAUNCH(h, false, reduce_final<<<1, 32, 0, h->stream>>>(h->d_diag, RED_BLOCKS, h->d_diag + RED_BLOCKS * NPART));
    DL_CUDA(h, cudaGetLastError());
    double r[NPART];
    DL_CUDA(h, cudaMemcpyAsync(r, h->d_diag + RED_BLOCKS * NPART, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    memset(out, 0, sizeof(*out));
    out->phi_sum = r[0];
    out->p_sum = r[1];
    out->mom[0] = r[2];
    out->mom[1] = r[3];
    out->mom[2] = r[4];
    out->ke = r[5];
    out->diss = r[6];
    out->vol_count = r[7];
    out->vol_smooth = r[8];
    out->p_in = r[9];
    out->n_in = r[10];
    out->p_out = r[11];
    out->n_out = r[12];
    out->w_sum = r[13];
    out->w_x[0] = r[14];
    out->w_x[1] = r[15];
    out->w_x[2] = r[16];
    out->w_xx[0] = r[17];
    out->w_xx[1] = r[18];
    out->w_xx[2] = r[19];
    out->w_xx[3] = r[20];
    out->w_xx[4] = r[21];
    out->w_xx[5] = r[22];
    out->phi_min = r[NSUM];
    out->phi_max = r[NSUM + 1];
    (void)r[23];
    return DL_OK;
}

int reduce_fields(dl_handle* h, const double* d_mac, dl_diag* out) { return reduce_any<double>(h, d_mac, 0.0, 0.0, out); }

int reduce_fields_f32(dl_handle* h, const float* d_mac, dl_diag* out) {
    return reduce_any<float>(h, d_mac, h->P.phi1, 1.0 / 3.0, out);
}

}  // namespace dl
