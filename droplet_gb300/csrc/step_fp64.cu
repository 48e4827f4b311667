// step_fp64.cu -- the plain form: FP64 storage and arithmetic, evaluated in
// the reference's order so that results are bitwise those of the FP64
// restatement (compiled here with --fmad=false; divisions and sqrt are the
// IEEE-rounded CUDA operators).
//
// One time step = two launches:
//   derive_fp64   per site: p0, lap(phi), grad(phi), G, the feq prefactor A,
//                 tau_g (and grad(u) when the LES or Anu terms need it);
//                 program/lbm_drop_xy.f90:590-666 and :576-587,
//                 program/LES_drop_xy.f90:481-502,663-690.
//   collide_fp64  per destination site: pull f_i, g_i from x - c_i, evaluate
//                 feq_i, geq_i at the source (equilibrium_cal :421-476),
//                 collide and add the force (fg_cal :478-515), apply the
//                 moving-wall bounce-back (drop8_mpi.f90:642-674), take the
//                 moments (physics :541-552) and reduce phi min/max
//                 (:559-574) with one atomic per block; the last block turns
//                 the reduction into the next step's tau_g range.
// On GB300 this form is bound by the FP64 pipe, not by HBM (about 1.7k FP64 flops per site).
#include "dl_internal.cuh"
#include "dl_device.cuh"

#include <string.h>
#include <math.h>

namespace dl {

struct Fp64Args {
    int nx, ny, nz;
    long long N;
    const double* f;   // [15][N]
    const double* g;
    double* fo;
    double* go;
    const double* mac;  // [5][N] phi,u1,u2,u3,p
    double* maco;
    double* rec;        // [nrec][N]
    const double* force;  // [3][N]
    DevState* st;
    double tauf, kf, kf6, kg, T, a, b, lapdiv, graddiv;
    double phi1, phi2, nu1, dnu, csd, anu23, anuds, ds;
    double F0;
    double E[Q], F[Q], Ekf[Q], Ekg[Q], ds3E[Q];
    double wall_bot[5], wall_top[5];  // 6 E_src (U . c_src) terms
    int walls;
    int visc_fixed;
    int les;
    long long step;
};

// record slots
enum { R_A = 0, R_TAUG = 1, R_G = 2, R_GU = 11 };


template <int AL>
__device__ __forceinline__ constexpr int cc(int i) {
    return AL == 0 ? cx(i) : (AL == 1 ? cy(i) : cz(i));
}

// sum_{i=1..14} c_{AL,i} v[i] in the reference's order (terms with c = 0 add
// a signed zero, which never changes a running sum that started at +0).
template <int AL>
__device__ __forceinline__ double csum(const double* v) {
    double s = 0.0;
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        if (cc<AL>(i) == 1) s = s + v[i];
        else if (cc<AL>(i) == -1) s = s - v[i];
    }
    return s;
}

// (cr1*u1 + cr2*u2) + cr3*u3 with zero terms dropped
__device__ __forceinline__ double cdot(int i, double u1, double u2, double u3) {
    double s = 0.0;
    bool any = false;
    if (cx(i) != 0) { s = cx(i) > 0 ? u1 : -u1; any = true; }
    if (cy(i) != 0) { double t = cy(i) > 0 ? u2 : -u2; s = any ? s + t : t; any = true; }
    if (cz(i) != 0) { double t = cz(i) > 0 ? u3 : -u3; s = any ? s + t : t; any = true; }
    return s;
}

// gtemp = sum_{be} sum_{al} G(al,be) c_al c_be, G(al,be) at rec[R_G + al + 3 be]
__device__ __forceinline__ double gcontract(int i, const double* __restrict__ rec, long long N, long long y) {
    if (i == 0) return 0.0;
    if (i <= 6) {
        int al = cx(i) != 0 ? 0 : (cy(i) != 0 ? 1 : 2);
        return __ldg(rec + (R_G + al + 3 * al) * N + y);
    }
    const int c[3] = {cx(i), cy(i), cz(i)};
    double s = 0.0;
#pragma unroll
    for (int be = 0; be < 3; ++be)
#pragma unroll
        for (int al = 0; al < 3; ++al) {
            double v = __ldg(rec + (R_G + al + 3 * be) * N + y);
            s = (c[al] * c[be] > 0) ? s + v : s - v;
        }
    return s;
}

// ftemp = sum_{be} sum_{al} (gu(be,al) + gu(al,be)) c_al c_be, gu(a,al) at rec[R_GU + a + 3 al]
__device__ __forceinline__ double ucontract(int i, const double* __restrict__ rec, long long N, long long y) {
    if (i == 0) return 0.0;
    const int c[3] = {cx(i), cy(i), cz(i)};
    double s = 0.0;
#pragma unroll
    for (int be = 0; be < 3; ++be)
#pragma unroll
        for (int al = 0; al < 3; ++al) {
            if (c[al] * c[be] == 0) continue;
            double v = __ldg(rec + (R_GU + be + 3 * al) * N + y) + __ldg(rec + (R_GU + al + 3 * be) * N + y);
            s = (c[al] * c[be] > 0) ? s + v : s - v;
        }
    return s;
}

// feq_i and geq_i at site y (equilibrium_cal, program/lbm_drop_xy.f90:452-469)
template <bool ANU>
__device__ __forceinline__ void equil_fp64(const Fp64Args& a, int i, long long y, double& feq, double& geq) {
    const long long N = a.N;
    const double ph = __ldg(a.mac + y);
    const double U1 = __ldg(a.mac + N + y), U2 = __ldg(a.mac + 2 * N + y), U3 = __ldg(a.mac + 3 * N + y);
    const double P = __ldg(a.mac + 4 * N + y);
    const double A = __ldg(a.rec + R_A * N + y);
    const double cu = (i == 0) ? 0.0 : cdot(i, U1, U2, U3);
    const double gt = gcontract(i, a.rec, N, y);
    if (i == 0) {
        feq = ph + a.F0 * A;
    } else {
        feq = (a.F[i] * A + ((a.E[i] * ph) * 3.0) * cu) + a.Ekf[i] * gt;
    }
    const double usq = (U1 * U1 + U2 * U2) + U3 * U3;
    double inner = (((3.0 * P) + (3.0 * cu)) + (4.5 * (cu * cu))) - (1.5 * usq);
    if (ANU) inner = inner + a.anuds * ucontract(i, a.rec, N, y);
    geq = a.E[i] * inner + a.Ekg[i] * gt;
}

__device__ __forceinline__ void site_xyz(long long s, int nx, int ny, int& x, int& y, int& z) {
    long long t = s / nx;
    x = (int)(s - t * nx);
    z = (int)(t / ny);
    y = (int)(t - (long long)z * ny);
}

// ---------------------------------------------------------------------------
template <bool GRADU>
__global__ void __launch_bounds__(256) derive_fp64(const Fp64Args a) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    int x, y, z;
    site_xyz(s, a.nx, a.ny, x, y, z);
    const long long N = a.N;
    long long nb[Q];
#pragma unroll
    for (int i = 1; i < Q; ++i)
        nb[i] = wrapi(x + cx(i), a.nx) + (long long)a.nx * (wrapi(y + cy(i), a.ny) + (long long)a.ny * wrapi(z + cz(i), a.nz));
    const double* phi = a.mac;
    double v[Q];
#pragma unroll
    for (int i = 1; i < Q; ++i) v[i] = __ldg(phi + nb[i]);
    const double fun = __ldg(phi + s);
    // various_cal :606-613
    const double p0 = fun * a.T / (1.0 - a.b * fun) - a.a * (fun * fun);
    double lap = -(14.0 * fun);
#pragma unroll
    for (int i = 1; i < Q; ++i) lap = lap + v[i];
    lap = lap / a.lapdiv;
    double gr[3];
    gr[0] = csum<0>(v) / a.graddiv;
    gr[1] = csum<1>(v) / a.graddiv;
    gr[2] = csum<2>(v) / a.graddiv;
    // gphi_cal :655-661
    const double gsq = (gr[0] * gr[0] + gr[1] * gr[1]) + gr[2] * gr[2];
#pragma unroll
    for (int be = 0; be < 3; ++be)
#pragma unroll
        for (int al = 0; al < 3; ++al) {
            double G = (4.5 * gr[al]) * gr[be];
            if (al == be) G = G - 1.5 * gsq;
            a.rec[(R_G + al + 3 * be) * N + s] = G;
        }
    // the bracket multiplying F(i) in feq (:453-456)
    a.rec[R_A * N + s] = (p0 - (a.kf * fun) * lap) - a.kf6 * gsq;
    // grad(u) (:623-633)
    double gu[9];
    if (GRADU) {
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            const double* uc = a.mac + (1 + comp) * N;
            double w[Q];
#pragma unroll
            for (int i = 1; i < Q; ++i) w[i] = __ldg(uc + nb[i]);
            gu[comp + 0] = csum<0>(w) / a.graddiv;
            gu[comp + 3] = csum<1>(w) / a.graddiv;
            gu[comp + 6] = csum<2>(w) / a.graddiv;
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) a.rec[(R_GU + k) * N + s] = gu[k];
    }
    // tau_g (:576-587; LES :663-690)
    double mn, mx;
    if (a.visc_fixed) {
        mn = a.phi1;
        mx = a.phi2;
    } else {
        mn = a.st->phi_min;
        mx = a.st->phi_max;
    }
    const double nu = (fun - mn) / (mx - mn) * a.dnu + a.nu1;
    double nue = 0.0;
    if (GRADU && a.les) {
        double acc = 0.0;
#pragma unroll
        for (int be = 0; be < 3; ++be)
#pragma unroll
            for (int al = 0; al < 3; ++al) {
                double st = 0.5 * (gu[al + 3 * be] + gu[be + 3 * al]);
                acc = acc + st * st;
            }
        nue = a.csd * sqrt(2.0 * acc);
    }
    a.rec[R_TAUG * N + s] = (0.5 + (3.0 * (nu + nue)) / a.ds) + a.anu23;
}

// ---------------------------------------------------------------------------
// initial populations f <- feq, g <- geq at the site itself (ini :248-251)
template <bool ANU>
__global__ void __launch_bounds__(256) equilibrium_fp64(const Fp64Args a) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= a.N) return;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        double fe, ge;
        equil_fp64<ANU>(a, i, s, fe, ge);
        if (a.fo) a.fo[i * a.N + s] = fe;
        a.go[i * a.N + s] = ge;
    }
}

// moments of the populations at each site (physics :541-552)
__device__ __forceinline__ void moments_fp64(const double* fn, const double* gn, double& ph, double& pp,
                                             double& a1, double& a2, double& a3) {
    ph = 0.0;
    pp = 0.0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        ph = ph + fn[i];
        pp = pp + gn[i] / 3.0;
    }
    a1 = 0.0;
    a2 = 0.0;
    a3 = 0.0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (cx(i) == 1) a1 = a1 + gn[i];
        else if (cx(i) == -1) a1 = a1 - gn[i];
        if (cy(i) == 1) a2 = a2 + gn[i];
        else if (cy(i) == -1) a2 = a2 - gn[i];
        if (cz(i) == 1) a3 = a3 + gn[i];
        else if (cz(i) == -1) a3 = a3 - gn[i];
    }
}

__global__ void __launch_bounds__(256) moments_kernel_fp64(const Fp64Args a) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    double fn[Q], gn[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        fn[i] = a.f ? a.f[i * a.N + s] : 0.0;
        gn[i] = a.g[i * a.N + s];
    }
    double ph, pp, a1, a2, a3;
    moments_fp64(fn, gn, ph, pp, a1, a2, a3);
    a.maco[s] = a.f ? ph : a.phi1;
    a.maco[a.N + s] = a1;
    a.maco[2 * a.N + s] = a2;
    a.maco[3 * a.N + s] = a3;
    a.maco[4 * a.N + s] = pp;
}

// ---------------------------------------------------------------------------
template <bool FORCE, bool ANU>
__global__ void __launch_bounds__(256) collide_fp64(const Fp64Args a) {
    const long long s0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool active = s0 < a.N;
    const long long s = active ? s0 : 0;
    const long long N = a.N;
    int x, y, z;
    site_xyz(s, a.nx, a.ny, x, y, z);
    double fn[Q], gn[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const long long src = wrapi(x - cx(i), a.nx) +
                              (long long)a.nx * (wrapi(y - cy(i), a.ny) + (long long)a.ny * wrapi(z - cz(i), a.nz));
        const double gs = __ldg(a.g + i * N + src);
        double fe, ge;
        equil_fp64<ANU>(a, i, src, fe, ge);
        if (a.f) {
            const double fs = __ldg(a.f + i * N + src);
            fn[i] = fs - (fs - fe) / a.tauf;
        } else {
            fn[i] = 0.0;  // single phase: no f
        }
        double gv = gs - (gs - ge) / __ldg(a.rec + R_TAUG * N + src);
        if (FORCE && i != 0) {
            const double cF = cdot(i, __ldg(a.force + src), __ldg(a.force + N + src), __ldg(a.force + 2 * N + src));
            gv = gv + a.ds3E[i] * cF;
        }
        gn[i] = gv;
    }
    if (a.walls) {
        // bounce_back_LBM, drop8_mpi.f90:651-671 (reference i = 4,8,9,10,15 <- 7,12,13,14,11
        // at the bottom; 7,11,12,13,14 <- 4,15,8,9,10 at the top)
        if (z == 0) {
            gn[3] = gn[6] - a.wall_bot[0];
            gn[7] = gn[11] - a.wall_bot[1];
            gn[8] = gn[12] - a.wall_bot[2];
            gn[9] = gn[13] - a.wall_bot[3];
            gn[14] = gn[10] - a.wall_bot[4];
        }
        if (z == a.nz - 1) {
            gn[6] = gn[3] - a.wall_top[0];
            gn[10] = gn[14] - a.wall_top[1];
            gn[11] = gn[7] - a.wall_top[2];
            gn[12] = gn[8] - a.wall_top[3];
            gn[13] = gn[9] - a.wall_top[4];
        }
    }
    double ph, pp, a1, a2, a3;
    moments_fp64(fn, gn, ph, pp, a1, a2, a3);
    if (!a.f) ph = a.phi1;
    bool bad = false;
    if (active) {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            if (a.f) a.fo[i * N + s] = fn[i];
            a.go[i * N + s] = gn[i];
        }
        a.maco[s] = ph;
        a.maco[N + s] = a1;
        a.maco[2 * N + s] = a2;
        a.maco[3 * N + s] = a3;
        a.maco[4 * N + s] = pp;
        bad = !(isfinite(ph) && isfinite(pp) && isfinite(a1) && isfinite(a2) && isfinite(a3));
    }
    // NaN is skipped by the reference's comparisons; exclude it here as well
    const double vmin = (active && ph == ph) ? ph : INFINITY;
    const double vmax = (active && ph == ph) ? ph : -INFINITY;
    minmax_block_and_finalize<double>(a.st, vmin, vmax, a.maco, 0.0, N, a.phi1, a.phi2, bad, a.step, gridDim.x);
}

// ---------------------------------------------------------------------------
static void fill_args(dl_handle* h, Fp64Args& a) {
    const dl_params& P = h->P;
    memset(&a, 0, sizeof(a));
    a.nx = h->nx;
    a.ny = h->ny;
    a.nz = h->nz;
    a.N = (long long)h->N;
    a.st = h->d_state;
    a.tauf = P.tauf;
    a.kf = P.kappaf;
    a.kf6 = P.kappaf / 6.0;
    a.kg = P.kappag;
    a.T = P.T;
    a.a = P.a;
    a.b = P.b;
    a.lapdiv = 5.0 * (P.ds * P.ds);
    a.graddiv = 10.0 * P.ds;
    a.phi1 = P.phi1;
    a.phi2 = P.phi2;
    a.nu1 = P.nu1;
    a.dnu = P.nu2 - P.nu1;
    a.csd = P.Cs * P.Cs * P.delta * P.delta;
    a.anu23 = (2.0 / 3.0) * P.Anu;
    a.anuds = P.Anu * P.ds;
    a.ds = P.ds;
    a.F0 = h->lc.F[0];
    for (int i = 0; i < Q; ++i) {
        a.E[i] = h->lc.E[i];
        a.F[i] = h->lc.F[i];
        a.Ekf[i] = h->lc.Ekf[i];
        a.Ekg[i] = h->lc.Ekg[i];
        a.ds3E[i] = h->lc.ds3E[i];
    }
    a.walls = P.walls ? 1 : 0;
    a.visc_fixed = (P.visc_mode == DL_VISC_FIXED) ? 1 : 0;
    a.les = P.les ? 1 : 0;
    a.rec = h->rec64;
    a.force = h->force64;
}

static inline unsigned nblocks(long long N, int bs) { return (unsigned)((N + bs - 1) / bs); }

int fp64_alloc(dl_handle* h) {
    const size_t N = h->N;
    const bool gradu = h->P.les || h->P.Anu != 0.0;
    h->nrec = gradu ? 20 : 11;
    for (int k = 0; k < 2; ++k) {
        if (!h->single) {  // the single-phase step has no f
            DL_CUDA(h, cudaMalloc(&h->f64[k], sizeof(double) * Q * N));
            DL_CUDA(h, cudaMemsetAsync(h->f64[k], 0, sizeof(double) * Q * N, h->stream));
        }
        DL_CUDA(h, cudaMalloc(&h->g64[k], sizeof(double) * Q * N));
        DL_CUDA(h, cudaMalloc(&h->mac64[k], sizeof(double) * 5 * N));
        DL_CUDA(h, cudaMemsetAsync(h->g64[k], 0, sizeof(double) * Q * N, h->stream));
        DL_CUDA(h, cudaMemsetAsync(h->mac64[k], 0, sizeof(double) * 5 * N, h->stream));
    }
    DL_CUDA(h, cudaMalloc(&h->rec64, sizeof(double) * h->nrec * N));
    DL_CUDA(h, cudaMalloc(&h->force64, sizeof(double) * 3 * N));
    DL_CUDA(h, cudaMemsetAsync(h->force64, 0, sizeof(double) * 3 * N, h->stream));
    return DL_OK;
}

void fp64_free(dl_handle* h) {
    for (int k = 0; k < 2; ++k) {
        cudaFree(h->f64[k]);
        cudaFree(h->g64[k]);
        cudaFree(h->mac64[k]);
        h->f64[k] = h->g64[k] = h->mac64[k] = nullptr;
    }
    cudaFree(h->rec64);
    cudaFree(h->force64);
    h->rec64 = h->force64 = nullptr;
}

static void launch_derive(dl_handle* h, const Fp64Args& a) {
    const bool gradu = h->P.les || h->P.Anu != 0.0;
    const unsigned nb = nblocks(a.N, 256);
    if (gradu) DL_LAUNCH(h, false, derive_fp64<true><<<nb, 256, 0, h->stream>>>(a));
    else DL_LAUNCH(h, false, derive_fp64<false><<<nb, 256, 0, h->stream>>>(a));
}

int fp64_init_equilibrium(dl_handle* h) {
    Fp64Args a;
    fill_args(h, a);
    a.mac = h->mac64[h->cur];
    a.fo = h->f64[h->cur];
    a.go = h->g64[h->cur];
    a.visc_fixed = 1;
    launch_derive(h, a);
    const unsigned nb = nblocks(a.N, 256);
    if (h->P.Anu != 0.0) DL_LAUNCH(h, false, equilibrium_fp64<true><<<nb, 256, 0, h->stream>>>(a));
    else DL_LAUNCH(h, false, equilibrium_fp64<false><<<nb, 256, 0, h->stream>>>(a));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int fp64_moments_from_populations(dl_handle* h) {
    Fp64Args a;
    fill_args(h, a);
    a.f = h->f64[h->cur];
    a.g = h->g64[h->cur];
    a.maco = h->mac64[h->cur];
    DL_LAUNCH(h, false, moments_kernel_fp64<<<nblocks(a.N, 256), 256, 0, h->stream>>>(a));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int fp64_step(dl_handle* h) {
    const int c = h->cur, n = 1 - c;
    const long long step = h->step + 1;
    if (h->force_mode == DL_FORCE_SPECTRAL) {
        int rc = spectral_force_fp64(h, h->mac64[c] + h->N, h->mac64[c] + 2 * h->N, h->mac64[c] + 3 * h->N,
                                     h->force64, h->force64 + h->N, h->force64 + 2 * h->N);
        if (rc != DL_OK) return rc;
    }
    Fp64Args a;
    fill_args(h, a);
    a.f = h->f64[c];
    a.g = h->g64[c];
    a.fo = h->f64[n];
    a.go = h->g64[n];
    a.mac = h->mac64[c];
    a.maco = h->mac64[n];
    a.step = step;
    // wall terms 6 E_src (U . c_src) in the reference's rounding (drop8_mpi.f90:652-670)
    double U[3] = {0.0, 0.0, 0.0};
    if (step >= h->P.wall_start)
        for (int k = 0; k < 3; ++k) U[k] = h->P.wall_u[k];
    const int bot_src[5] = {6, 11, 12, 13, 10}, top_src[5] = {3, 14, 7, 8, 9};
    for (int k = 0; k < 5; ++k) {
        int j = bot_src[k];
        a.wall_bot[k] = 6.0 * h->lc.E[j] * ((-U[0]) * (double)cx(j) + (-U[1]) * (double)cy(j) + (-U[2]) * (double)cz(j));
        j = top_src[k];
        a.wall_top[k] = 6.0 * h->lc.E[j] * ((U[0]) * (double)cx(j) + (U[1]) * (double)cy(j) + (U[2]) * (double)cz(j));
    }
    launch_derive(h, a);
    const unsigned nb = nblocks(a.N, 256);
    const bool force = h->force_mode != DL_FORCE_NONE;
    const bool anu = h->P.Anu != 0.0;
    if (force) {
        if (anu) DL_LAUNCH(h, true, collide_fp64<true, true><<<nb, 256, 0, h->stream>>>(a));
        else DL_LAUNCH(h, true, collide_fp64<true, false><<<nb, 256, 0, h->stream>>>(a));
    } else {
        if (anu) DL_LAUNCH(h, true, collide_fp64<false, true><<<nb, 256, 0, h->stream>>>(a));
        else DL_LAUNCH(h, true, collide_fp64<false, false><<<nb, 256, 0, h->stream>>>(a));
    }
    DL_CUDA(h, cudaGetLastError());
    h->cur = n;
    h->step = step;
    return DL_OK;
}

}  // namespace dl
