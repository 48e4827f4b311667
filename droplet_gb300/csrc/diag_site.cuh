// diag_site.cuh -- the per-site terms of the whole-domain diagnostics that
// dl_reduce and dl_reduce_static sum (one definition for both):
// conservation sums (phi, p, momentum), kinetic energy, dissipation
// 2 nu(phi) S:S with the reference's 14-neighbour gradient stencil
// (program/lbm_drop_xy.f90:615-633; dissipation convention of
// program/energy_budget.f90:1494), droplet volume (phi above the mid value,
// threshold of program/percolation.f90:112), pressure inside and outside,
// and the moments of w = (phi - phi1)/(phi2 - phi1) for the deformation D
// (prototype_program/two-phase/drop8_mpi.f90:812-970), FP64 throughout.
//
// The stencil weights are -1, 0, +1, so the gradient is formed by signed
// additions only (a product with a zero weight is never issued); it and the
// strain contraction S:S (over the six distinct entries of the symmetric
// strain) are formed in the storage type of the fields (FP32 for the FP32 and
// FP16 forms, as their step forms the LES strain; FP64 for the FP64 form),
// then scaled by 1/(4 graddiv^2) in FP64: GB300's FP64 pipe is narrow.
#pragma once

#include "dl_internal.cuh"
#include "dl_device.cuh"

namespace dl {

constexpr int DIAG_NSUM = 24;  // sums; then min and max of phi

struct DiagConsts {
    int nx, ny, nz;
    long long N;
    double phi1, phi_off, p_off;  // stored phi and p are phi - phi_off, p - p_off
    double inv_span, mid, nu1, dnu;
    double sfac;  // 1 / (4 graddiv^2)
};

// the constants for handle h (reduce.cu)
void diag_consts(const dl_handle* h, double phi_off, double p_off, DiagConsts& k);

__device__ __forceinline__ int diag_wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// site s = x + nx (y + ny z): add its terms to acc, fold phi into [vmin, vmax]
template <typename T>
__device__ __forceinline__ void diag_site(const T* __restrict__ mac, const DiagConsts& k, long long s, int x, int y,
                                          int z, double (&acc)[DIAG_NSUM], double& vmin, double& vmax) {
    const long long N = k.N;
    const double ph = k.phi_off + (double)mac[s];
    const double u1 = (double)mac[N + s], u2 = (double)mac[2 * N + s], u3 = (double)mac[3 * N + s];
    const double p = k.p_off + (double)mac[4 * N + s];
    long long xo[3], yo[3], zo[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        xo[d] = diag_wrap(x - 1 + d, k.nx);
        yo[d] = (long long)k.nx * diag_wrap(y - 1 + d, k.ny);
        zo[d] = (long long)k.nx * k.ny * diag_wrap(z - 1 + d, k.nz);
    }
    // du_b/dx_a: g[b + 3 a]
    T g[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) g[j] = T(0);
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const long long nb = xo[1 + cx(i)] + yo[1 + cy(i)] + zo[1 + cz(i)];
        const T v[3] = {mac[N + nb], mac[2 * N + nb], mac[3 * N + nb]};
        const int c[3] = {cx(i), cy(i), cz(i)};
#pragma unroll
        for (int al = 0; al < 3; ++al)
#pragma unroll
            for (int be = 0; be < 3; ++be) {
                if (c[al] > 0) g[be + 3 * al] += v[be];
                else if (c[al] < 0) g[be + 3 * al] -= v[be];
            }
    }
    // S:S before the scale, in the storage type (for FP64 fields the FP64 expression)
    const T d01 = g[1] + g[3], d02 = g[2] + g[6], d12 = g[5] + g[7];
    const T sT = T(4) * (g[0] * g[0] + g[4] * g[4] + g[8] * g[8]) + T(2) * (d01 * d01 + d02 * d02 + d12 * d12);
    const double ss = k.sfac * (double)sT;
    const double w = (ph - k.phi1) * k.inv_span;
    const double nu = k.nu1 + w * k.dnu;
    acc[0] += ph;
    acc[1] += p;
    acc[2] += u1;
    acc[3] += u2;
    acc[4] += u3;
    acc[5] += 0.5 * (u1 * u1 + u2 * u2 + u3 * u3);
    acc[6] += 2.0 * nu * ss;
    acc[7] += (ph > k.mid) ? 1.0 : 0.0;
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

// this thread's sites s0, s0 + stride, ... below N with their (x, y, z)
// advanced incrementally (one 64-bit division per thread)
template <typename T>
__device__ __forceinline__ void diag_sites(const T* __restrict__ mac, const DiagConsts& k, long long s0,
                                           long long stride, double (&acc)[DIAG_NSUM], double& vmin,
                                           double& vmax) {
    if (s0 >= k.N) return;
    const long long nxy = (long long)k.nx * k.ny;
    long long z = s0 / nxy;
    long long r = s0 - z * nxy;
    int y = (int)(r / k.nx), x = (int)(r - (long long)y * k.nx);
    const long long dz = stride / nxy, rr = stride - dz * nxy;
    const int dy = (int)(rr / k.nx), dx = (int)(rr - (long long)dy * k.nx);
    for (long long s = s0; s < k.N; s += stride) {
        diag_site(mac, k, s, x, y, (int)z, acc, vmin, vmax);
        x += dx;
        if (x >= k.nx) {
            x -= k.nx;
            ++y;
        }
        y += dy;
        if (y >= k.ny) {
            y -= k.ny;
            ++z;
        }
        z += dz;
    }
}

}  // namespace dl
