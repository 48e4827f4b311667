// reduce.cu -- FP64 whole-domain diagnostics of the macroscopic fields:
// conservation sums (phi, p, momentum), kinetic energy, dissipation
// 2 nu(phi) S:S with the reference's 14-neighbour gradient stencil
// (program/lbm_drop_xy.f90:615-633; dissipation convention of
// program/energy_budget.f90:1494), droplet volume (phi above the mid value,
// threshold of program/percolation.f90:112) and the second-moment tensor of
// w = (phi - phi1)/(phi2 - phi1) for the deformation D (the inertia tensor of
// prototype_program/two-phase/drop8_mpi.f90:812-970, taken over the volume).
//
// Two launches: per-block partial sums (one pass over the fields, per-thread
// FP64 accumulators, warp-shuffle then shared-memory tree), then one warp
// that adds the partials of every block in a fixed order with Neumaier
// compensation, so the result is deterministic.
#include "dl_internal.cuh"

#include <string.h>

namespace dl {

constexpr int NSUM = 24;  // sums, then min, max
constexpr int NPART = NSUM + 2;
constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs
constexpr int RED_THREADS = 256;

struct RedArgs {
    int nx, ny, nz;
    long long N;
    double phi1, phi2, nu1, dnu, graddiv;
    double phi_off, p_off;  // stored phi and p are phi - phi_off, p - p_off
    double* part;
};

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) reduce_partials(const T* __restrict__ mac, const RedArgs a) {
    double acc[NSUM];
#pragma unroll
    for (int k = 0; k < NSUM; ++k) acc[k] = 0.0;
    double vmin = INFINITY, vmax = -INFINITY;
    const long long N = a.N;
    const double inv = 1.0 / (a.phi2 - a.phi1);
    const double mid = 0.5 * (a.phi1 + a.phi2);
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
        const long long t = s / a.nx;
        const int x = (int)(s - t * a.nx);
        const int z = (int)(t / a.ny);
        const int y = (int)(t - (long long)z * a.ny);
        const double ph = a.phi_off + (double)mac[s];
        const double u1 = (double)mac[N + s], u2 = (double)mac[2 * N + s], u3 = (double)mac[3 * N + s];
        const double p = a.p_off + (double)mac[4 * N + s];
        // velocity gradient with the 14-neighbour stencil
        double gu[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) gu[k] = 0.0;
#pragma unroll
        for (int i = 1; i < Q; ++i) {
            const int xx = x + cx(i), yy = y + cy(i), zz = z + cz(i);
            const long long nb = (xx < 0 ? xx + a.nx : (xx >= a.nx ? xx - a.nx : xx)) +
                                 (long long)a.nx * ((yy < 0 ? yy + a.ny : (yy >= a.ny ? yy - a.ny : yy)) +
                                                    (long long)a.ny * (zz < 0 ? zz + a.nz : (zz >= a.nz ? zz - a.nz : zz)));
            const double v1 = (double)mac[N + nb], v2 = (double)mac[2 * N + nb], v3 = (double)mac[3 * N + nb];
            const double c[3] = {(double)cx(i), (double)cy(i), (double)cz(i)};
#pragma unroll
            for (int al = 0; al < 3; ++al) {
                gu[0 + 3 * al] += c[al] * v1;
                gu[1 + 3 * al] += c[al] * v2;
                gu[2 + 3 * al] += c[al] * v3;
            }
        }
        double ss = 0.0;
#pragma unroll
        for (int be = 0; be < 3; ++be)
#pragma unroll
            for (int al = 0; al < 3; ++al) {
                const double st = 0.5 * (gu[al + 3 * be] + gu[be + 3 * al]) / a.graddiv;
                ss += st * st;
            }
        const double w = (ph - a.phi1) * inv;
        const double nu = a.nu1 + w * a.dnu;
        acc[0] += ph;
        acc[1] += p;
        acc[2] += u1;
        acc[3] += u2;
        acc[4] += u3;
        acc[5] += 0.5 * (u1 * u1 + u2 * u2 + u3 * u3);
        acc[6] += 2.0 * nu * ss;
        acc[7] += (ph > mid) ? 1.0 : 0.0;
        acc[8] += w;
        if (w > 0.95) {
            acc[9] += p;
            acc[10] += 1.0;
        }
        if (w < 0.05) {
            acc[11] += p;
            acc[12] += 1.0;
        }
        const double X = (double)x, Y = (double)y, Z = (double)z;
        acc[13] += w;
        acc[14] += w * X;
        acc[15] += w * Y;
        acc[16] += w * Z;
        acc[17] += w * X * X;
        acc[18] += w * Y * Y;
        acc[19] += w * Z * Z;
        acc[20] += w * X * Y;
        acc[21] += w * X * Z;
        acc[22] += w * Y * Z;
        acc[23] += (ph == ph && isfinite(ph)) ? 0.0 : 1.0;
        if (ph == ph) {
            vmin = fmin(vmin, ph);
            vmax = fmax(vmax, ph);
        }
    }
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

template <typename T>
static int reduce_any(dl_handle* h, const T* d_mac, double phi_off, double p_off, dl_diag* out) {
    if (!h->d_diag) DL_CUDA(h, cudaMalloc(&h->d_diag, sizeof(double) * (RED_BLOCKS * NPART + NPART)));
    RedArgs a;
    memset(&a, 0, sizeof(a));
    a.nx = h->nx;
    a.ny = h->ny;
    a.nz = h->nz;
    a.N = (long long)h->N;
    a.phi1 = h->P.phi1;
    a.phi2 = h->P.phi2;
    a.nu1 = h->P.nu1;
    a.dnu = h->P.nu2 - h->P.nu1;
    a.graddiv = 10.0 * h->P.ds;
    a.phi_off = phi_off;
    a.p_off = p_off;
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
