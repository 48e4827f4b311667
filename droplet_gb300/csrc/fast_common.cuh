// fast_common.cuh -- device code shared by the reduced-precision step kernels:
// the pull form (step_fast.cu, collision at the source by the destination
// thread) and the push form (step_push.cu, collision by the source's own
// thread, streamed by the store): the step arguments, the D3Q15 weights in
// FP32, the per-site record (p0, stencils, eddy viscosity), the storage
// policies of the FP32 and FP16 forms, and the band forcing's projection
// and finalisation.
#pragma once
#include "dl_internal.cuh"
#include "dl_device.cuh"

#include <cuda_fp16.h>
#include <math.h>
#include <string.h>
#include <algorithm>
#include <vector>

namespace dl {

constexpr int TX = 32, TY = 8, NT = TX * TY, NWARP = NT / 32;
constexpr int EX1 = TX + 2, EY1 = TY + 2, P1 = EX1 * EY1;  // record plane (1-cell halo)
constexpr int EX2 = TX + 4, EY2 = TY + 4, P2 = EX2 * EY2;  // staging plane (2-cell halo)
enum { R_DPHI, R_U1, R_U2, R_U3, R_DA, R_S, R_OMG, R_GX, R_GY, R_GZ, R_NBASE };

enum { F_NONE = 0, F_ARRAY = 1, F_SPECTRAL = 2 };
constexpr int SK = 2;                 // in-kernel spectral forcing: |k_x| <= 2 (kc <= 3)
constexpr int SNK = 2 * SK + 1;
constexpr int SMAXM = 64;             // at most 64 band modes (two per lane)
constexpr int SP_NREP = 4;            // copies of the projection accumulators (block b adds to copy b % 4)

struct FastArgs {
    int nx, ny, nz, lz;
    int l2_prefetch;
    int proj_in_step;  // band projection of the new u at the end of the fused step (F_SPECTRAL)
    long long N;
    const float* mac;  // [5][N] dphi, u1, u2, u3, dp
    float* maco;
    const void* f;     // [15][N] storage
    const void* g;
    void* fo;
    void* go;
    const float* force;  // [3][N] (F_ARRAY)
    DevState* st;
    float phi1, phi2, omf, kf, kf6, kg, T, a, b, omb1, nu1, dnu, csd, anu23, inv_ds, inv_lap, inv_grad;
    float omg_sp;  // 1/tau_g of the single-phase step, tau_g = 1/2 + 3 nu1/ds
    float fref[Q];   // bulk equilibrium of f (FP32 form offsets)
    float wall_bot[5], wall_top[5];
    int walls, visc_fixed;
    long long step;
    // in-kernel spectral forcing (F_SPECTRAL)
    int nm;               // number of band modes (half spectrum kz >= 0)
    const int4* modes;    // kx, ky, kz, weight; sorted by kx
    const int* kx_off;    // [SNK + 1] first mode of each kx = -2..2
    const float2* fh;     // [3][nm] w * (0.5 eps / E) * u_hat, used by this step
    float2* fh_next;      // [3][nm] written by the last block
    double* acc;          // [3][nm][2] sum over sites of u e^{-i k.x} of the new u
    const float2* twx;    // e^{+i 2 pi m / n}
    const float2* twy;
    const float2* twz;
    double half_eps, invN;
};

// v within a few periods of [0, n) (plane indices z - 2 .. z + 4): no division
__device__ __forceinline__ int wrap_near(int v, int n) {
    while (v < 0) v += n;
    while (v >= n) v -= n;
    return v;
}

__device__ __forceinline__ int pmod(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}

// ---- lattice constants in FP32 -------------------------------------------
__device__ __forceinline__ constexpr float Ew(int i) { return i == 0 ? 2.0f / 9.0f : (i <= 6 ? 1.0f / 9.0f : 1.0f / 72.0f); }
__device__ __forceinline__ constexpr float Fw(int i) { return i == 0 ? -7.0f / 3.0f : (i <= 6 ? 1.0f / 3.0f : 1.0f / 24.0f); }
__device__ __forceinline__ constexpr float c2w(int i) { return i == 0 ? 0.f : (i <= 6 ? 1.f : 3.f); }

// x times a lattice constant c given exactly (in double) as the pair hi + lo of
// floats: one rounding of the exact product, with no bias. A constant such as
// 3 E_i = 1/3 rounded to one float is 3e-8 too large, the same at every site and
// step; in the odd part of an equilibrium that scales sum_i c_i geq_i = u by
// the same factor at every collision, and the error of u and of the phi flux
// then grows linearly with the steps instead of as a random walk.
__device__ __forceinline__ constexpr float c_hi(double c) { return (float)c; }
__device__ __forceinline__ constexpr float c_lo(double c) { return (float)(c - (double)(float)c); }
__device__ __forceinline__ float mulc(float x, double c) { return __fmaf_rn(x, c_hi(c), __fmul_rn(x, c_lo(c))); }
// exact D3Q15 constants by class (0 rest, 1 axis, 2 diagonal)
__device__ __forceinline__ constexpr double Ed(int c) { return c == 0 ? 2.0 / 9.0 : (c == 1 ? 1.0 / 9.0 : 1.0 / 72.0); }
__device__ __forceinline__ constexpr double Fd(int c) { return c == 0 ? -7.0 / 3.0 : (c == 1 ? 1.0 / 3.0 : 1.0 / 24.0); }

// c_i . (p, q, r) with the zero terms dropped; explicit roundings so that the
// same inputs give the same bits wherever it is inlined
__device__ __forceinline__ float cdot3(int i, float p, float q, float r) {
    float s = 0.f;
    bool any = false;
    if (cx(i) != 0) {
        s = cx(i) > 0 ? p : -p;
        any = true;
    }
    if (cy(i) != 0) {
        const float t = cy(i) > 0 ? q : -q;
        s = any ? __fadd_rn(s, t) : t;
        any = true;
    }
    if (cz(i) != 0) {
        const float t = cz(i) > 0 ? r : -r;
        s = any ? __fadd_rn(s, t) : t;
    }
    return s;
}

template <int AL>
__device__ __forceinline__ float csumf(const float* v) {
    float s = 0.f;
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const int c = AL == 0 ? cx(i) : (AL == 1 ? cy(i) : cz(i));
        if (c == 1) s += v[i];
        else if (c == -1) s -= v[i];
    }
    return s;
}

// p0(phi) - p0(phi1) without cancellation:
// dphi [T / ((1 - b phi)(1 - b phi1)) - a (phi + phi1)]. Every operation is
// rounded explicitly, so the writer and the reader of the FP16 residual basis
// (RES) get the same bits; RES takes the approximate reciprocal (deterministic;
// den lies in (0.3, 1) for the reference parameter sets), which made the FP16
// step 1.3 % faster and the FP32 step slower, so FP32 keeps the rounded one
template <bool RES>
__device__ __forceinline__ float site_dp0(const FastArgs& a, float dphi) {
    const float phi = __fadd_rn(a.phi1, dphi);
    const float den = __fmul_rn(__fmaf_rn(-a.b, phi, 1.f), a.omb1);
    const float t = __fmul_rn(a.T, RES ? __fdividef(1.f, den) : __frcp_rn(den));
    return __fmul_rn(dphi, __fmaf_rn(-a.a, __fadd_rn(phi, a.phi1), t));
}

__device__ __forceinline__ float site_S(float dp, float u1, float u2, float u3) {
    const float usq = __fmaf_rn(u3, u3, __fmaf_rn(u2, u2, __fmul_rn(u1, u1)));
    return __fmaf_rn(-1.5f, usq, __fmul_rn(3.f, dp));
}

// local part of the equilibria (the FP16 residual basis), deviation form; the
// lattice constants multiply as exact pairs (mulc): the basis is part of every
// post-collision value, so a biased constant would bias the fluxes (FP16 form,
// config 2: phi~ error 1.1e-3 -> 2.8e-4 after 2000 steps, for 5 % of its time)
__device__ __forceinline__ float fbar(int i, float dphi, float phi, float dp0, float cu) {
    if (i == 0) return __fadd_rn(dphi, mulc(dp0, Fd(0)));
    return __fadd_rn(mulc(__fmul_rn(phi, cu), 3.0 * Ed(wclass(i))), mulc(dp0, Fd(wclass(i))));
}
__device__ __forceinline__ float gbar(int i, float S, float cu) {
    return mulc(__fmaf_rn(cu, __fmaf_rn(4.5f, cu, 3.f), S), Ed(wclass(i)));
}

// ---- storage policies ----------------------------------------------------
template <typename ST>
struct Pop;
template <>
struct Pop<float> {
    static __device__ __forceinline__ float ld(const void* p, long long i) { return __ldg((const float*)p + i); }
    static __device__ __forceinline__ void st(void* p, long long i, float v) { ((float*)p)[i] = v; }
};
template <>
struct Pop<__half> {
    static __device__ __forceinline__ float ld(const void* p, long long i) {
        return __half2float(__ldg((const __half*)p + i));
    }
    static __device__ __forceinline__ void st(void* p, long long i, float v) { ((__half*)p)[i] = __float2half_rn(v); }
};

// ---- packed FP32x2 stencil sums (two staged fields per 64-bit word) -------------
// sum_{i=1..14} c_{AL,i} v[i] for both lanes: FADD2 for +1, FFMA2 with -1 for -1
template <int AL>
__device__ __forceinline__ float2 csum2(const float2* v) {
    float2 s = make_float2(0.f, 0.f);
    const float2 m1 = make_float2(-1.f, -1.f);
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const int c = AL == 0 ? cx(i) : (AL == 1 ? cy(i) : cz(i));
        if (c == 1) s = __fadd2_rn(s, v[i]);
        else if (c == -1) s = __ffma2_rn(v[i], m1, s);
    }
    return s;
}

// ---- the per-site record ------------------------------------------------------
struct Rec {
    float dphi, u1, u2, u3, dA, S, omg, gx, gy, gz, gsq, dp0, Fx, Fy, Fz;
    float gq;  // 1.5 |grad phi|^2 (stored records of the FP32 form)
};

// v[1..14]: dphi at the D3Q15 neighbours; w[c][1..14]: u_c there (LES only)
template <bool LES, bool RES>
__device__ __forceinline__ Rec make_record(const FastArgs& a, float dphi, const float* v, const float (*w)[Q],
                                           float u1, float u2, float u3, float dp, float mn, float kscale) {
    Rec r;
    float lap = -14.f * dphi;
#pragma unroll
    for (int i = 1; i < Q; ++i) lap += v[i];
    lap *= a.inv_lap;
    r.gx = csumf<0>(v) * a.inv_grad;
    r.gy = csumf<1>(v) * a.inv_grad;
    r.gz = csumf<2>(v) * a.inv_grad;
    r.gsq = r.gx * r.gx + r.gy * r.gy + r.gz * r.gz;
    const float phi = __fadd_rn(a.phi1, dphi);
    r.dp0 = site_dp0<RES>(a, dphi);
    r.dA = r.dp0 - a.kf * phi * lap - a.kf6 * r.gsq;
    r.dphi = dphi;
    r.u1 = u1;
    r.u2 = u2;
    r.u3 = u3;
    r.S = site_S(dp, u1, u2, u3);
    const float nu = (phi - mn) * kscale + a.nu1;  // kscale = dnu / (phi_max - phi_min), per block
    float nut = 0.f;
    if (LES) {
        float gu[9];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            gu[c + 0] = csumf<0>(w[c]) * a.inv_grad;
            gu[c + 3] = csumf<1>(w[c]) * a.inv_grad;
            gu[c + 6] = csumf<2>(w[c]) * a.inv_grad;
        }
        // S:S with S = (grad u + grad u^T)/2
        const float sxy = 0.5f * (gu[0 + 3 * 1] + gu[1 + 3 * 0]);
        const float sxz = 0.5f * (gu[0 + 3 * 2] + gu[2 + 3 * 0]);
        const float syz = 0.5f * (gu[1 + 3 * 2] + gu[2 + 3 * 1]);
        const float ss = gu[0] * gu[0] + gu[4] * gu[4] + gu[8] * gu[8] + 2.f * (sxy * sxy + sxz * sxz + syz * syz);
        const float t = 2.f * ss;
        nut = t > 0.f ? a.csd * (t * rsqrtf(t)) : 0.f;
    }
    r.omg = __fdividef(1.f, 0.5f + 3.f * (nu + nut) * a.inv_ds + a.anu23);  // tau_g >= 0.5 and far below 2^126, where the approximate division is within 2 ulp
    r.Fx = r.Fy = r.Fz = 0.f;
    return r;
}

// the LES record from pairs (phi - phi1, u1) and (u2, u3) at the 14 neighbours:
// the same sums as make_record<true>, two fields per packed instruction
template <bool RES>
__device__ __forceinline__ Rec make_record_les2(const FastArgs& a, float dphi, const float2* pa, const float2* pb,
                                                float u1, float u2, float u3, float dp, float mn, float kscale) {
    Rec r;
    float lap = -14.f * dphi;
#pragma unroll
    for (int i = 1; i < Q; ++i) lap += pa[i].x;
    lap *= a.inv_lap;
    const float2 ax = csum2<0>(pa), ay = csum2<1>(pa), az = csum2<2>(pa);  // (d phi, d u1)
    const float2 bx = csum2<0>(pb), by = csum2<1>(pb), bz = csum2<2>(pb);  // (d u2, d u3)
    r.gx = ax.x * a.inv_grad;
    r.gy = ay.x * a.inv_grad;
    r.gz = az.x * a.inv_grad;
    r.gsq = r.gx * r.gx + r.gy * r.gy + r.gz * r.gz;
    const float phi = __fadd_rn(a.phi1, dphi);
    r.dp0 = site_dp0<RES>(a, dphi);
    r.dA = r.dp0 - a.kf * phi * lap - a.kf6 * r.gsq;
    r.dphi = dphi;
    r.u1 = u1;
    r.u2 = u2;
    r.u3 = u3;
    r.S = site_S(dp, u1, u2, u3);
    const float nu = (phi - mn) * kscale + a.nu1;
    // gu[c + 3 al] = d u_c / d x_al
    float gu[9];
    gu[0] = ax.y * a.inv_grad;
    gu[3] = ay.y * a.inv_grad;
    gu[6] = az.y * a.inv_grad;
    gu[1] = bx.x * a.inv_grad;
    gu[4] = by.x * a.inv_grad;
    gu[7] = bz.x * a.inv_grad;
    gu[2] = bx.y * a.inv_grad;
    gu[5] = by.y * a.inv_grad;
    gu[8] = bz.y * a.inv_grad;
    const float sxy = 0.5f * (gu[0 + 3 * 1] + gu[1 + 3 * 0]);
    const float sxz = 0.5f * (gu[0 + 3 * 2] + gu[2 + 3 * 0]);
    const float syz = 0.5f * (gu[1 + 3 * 2] + gu[2 + 3 * 1]);
    const float ss = gu[0] * gu[0] + gu[4] * gu[4] + gu[8] * gu[8] + 2.f * (sxy * sxy + sxz * sxz + syz * syz);
    const float t = 2.f * ss;
    const float nut = t > 0.f ? a.csd * (t * rsqrtf(t)) : 0.f;
    r.omg = __fdividef(1.f, 0.5f + 3.f * (nu + nut) * a.inv_ds + a.anu23);  // tau_g >= 0.5 and far below 2^126, where the approximate division is within 2 ulp
    r.Fx = r.Fy = r.Fz = 0.f;
    return r;
}

// collide direction i at its source with record r; fin/gin are the stored values
template <bool RES, bool FORCE>
__device__ __forceinline__ void collide_dir(const FastArgs& a, int i, const Rec& r, float fin, float gin, float& fo,
                                            float& go) {
    const float phi = __fadd_rn(a.phi1, r.dphi);
    const float cu = (i == 0) ? 0.f : cdot3(i, r.u1, r.u2, r.u3);
    const float cg = (i == 0) ? 0.f : cdot3(i, r.gx, r.gy, r.gz);
    const float cGc = RES ? 4.5f * cg * cg - 1.5f * c2w(i) * r.gsq : (4.5f * cg) * cg - c2w(i) * r.gq;
    const float E = Ew(i);
    if (!RES) {
        const float dfeq = (i == 0 ? r.dphi : 0.f) + mulc(r.dA, Fd(wclass(i))) +
                           mulc(3.f * phi * cu + a.kf * cGc, Ed(wclass(i)));
        const float dgeq = mulc(r.S + cu * (3.f + 4.5f * cu) + a.kg * cGc, Ed(wclass(i)));
        fo = fin + a.omf * (dfeq - fin);
        go = gin + r.omg * (dgeq - gin);
    } else {
        const float fb = fbar(i, r.dphi, phi, r.dp0, cu);
        const float gb = gbar(i, r.S, cu);
        const float df = mulc(r.dA - r.dp0, Fd(wclass(i))) + mulc(a.kf * cGc, Ed(wclass(i)));
        fo = fb + fin + a.omf * (df - fin);
        go = gb + gin + r.omg * (mulc(a.kg * cGc, Ed(wclass(i))) - gin);
    }
    if (FORCE && i != 0) go += 3.f * E * cdot3(i, r.Fx, r.Fy, r.Fz);
}

// single-phase collision of g_i at its source (g_cal, program/lbm_iht_xy.f90:561-590):
// the two-phase rule without the interface terms
template <bool RES, bool FORCE>
__device__ __forceinline__ float collide_g(int i, float S, float omg, float u1, float u2, float u3, float Fx,
                                           float Fy, float Fz, float gin) {
    const float cu = (i == 0) ? 0.f : cdot3(i, u1, u2, u3);
    const float E = Ew(i);
    float go;
    if (!RES) {
        const float dgeq = mulc(S + cu * (3.f + 4.5f * cu), Ed(wclass(i)));
        go = gin + omg * (dgeq - gin);
    } else {
        go = gbar(i, S, cu) + gin + omg * (0.f - gin);
    }
    if (FORCE && i != 0) go += 3.f * E * cdot3(i, Fx, Fy, Fz);
    return go;
}

// shared scratch of spectral_finalize (doubles)
constexpr int FIN_SCRATCH = 6 * SMAXM + SMAXM + NWARP + 1;

// last block: band energy E = sum_m 0.5 w_m |u_hat_m|^2, u_hat = acc / N, and
// the coefficients w_m (0.5 eps / E) u_hat_m of the next step; zeroes acc.
// The folded sums stay in shared memory (scratch: FIN_SCRATCH doubles), so the
// block reads acc once.
static __device__ void spectral_finalize(const FastArgs& a, double* scratch) {
    double* s_acc = scratch;
    double* s_w = s_acc + 6 * SMAXM;
    double* s_e = s_w + SMAXM;
    double& s_coef = s_e[NWARP];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nv = 6 * a.nm;  // values per accumulator copy
    if (tid < a.nm) s_w[tid] = (double)__ldg(a.modes + tid).w;
    // fold the copies (fixed order), zero them: a thread's (at most two, nv <= 6 SMAXM
    // <= 2 blockDim.x) values in one pass, all loads in flight together
    static_assert(6 * SMAXM <= 2 * NT, "two folded values per thread");
    {
        double c[2][SP_NREP];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int t = tid + j * blockDim.x;
#pragma unroll
            for (int r = 0; r < SP_NREP; ++r) c[j][r] = t < nv ? __ldcg(a.acc + (size_t)r * nv + t) : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int t = tid + j * blockDim.x;
            if (t >= nv) continue;
            double v = c[j][0];
#pragma unroll
            for (int r = 1; r < SP_NREP; ++r) v += c[j][r];
#pragma unroll
            for (int r = 0; r < SP_NREP; ++r) a.acc[(size_t)r * nv + t] = 0.0;
            s_acc[t] = v;
        }
    }
    __syncthreads();
    double e = 0.0;
    for (int m = tid; m < a.nm; m += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double re = s_acc[2 * (c * a.nm + m)] * a.invN;
            const double im = s_acc[2 * (c * a.nm + m) + 1] * a.invN;
            s += re * re + im * im;
        }
        e += 0.5 * s_w[m] * s;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if (lane == 0) s_e[warp] = e;
    __syncthreads();
    if (tid == 0) {
        double E = 0.0;
        for (int w = 0; w < NWARP; ++w) E += s_e[w];
        s_coef = a.half_eps / E;
        a.st->sp_energy = E;
        a.st->sp_coef = s_coef;
    }
    __syncthreads();
    const double coef = s_coef;
    for (int t = tid; t < 3 * a.nm; t += blockDim.x) {
        const int m = t % a.nm;
        const double k = coef * a.invN * s_w[m];
        a.fh_next[t] = make_float2((float)(k * s_acc[2 * t]), (float)(k * s_acc[2 * t + 1]));
    }
}

// the tile's halo-indexed twiddle tables: s_tx[kx][ex] = (cos kx x, -sin kx x),
// s_ty[ky][ey] = e^{i ky y}, x = x0 - 1 + ex, y = y0 - 1 + ey
__device__ __forceinline__ void tile_twiddles(const FastArgs& a, float2* s_tx, float2* s_ty, int x0, int y0) {
    for (int t = threadIdx.x; t < SNK * EX1; t += NT) {
        const int kxi = t / EX1, ex = t % EX1;
        const float2 e = a.twx[pmod((kxi - SK) * pmod(x0 - 1 + ex, a.nx), a.nx)];
        s_tx[t] = make_float2(e.x, -e.y);  // Re(C e^{i kx x}) = C . (cos, -sin)
    }
    for (int t = threadIdx.x; t < SNK * EY1; t += NT) {
        const int kyi = t / EY1, ey = t % EY1;
        s_ty[t] = a.twy[pmod((kyi - SK) * pmod(y0 - 1 + ey, a.ny), a.ny)];
    }
}

// ---- band projection of the block's own tile, after its z march -----------------
// acc[c][m] += sum over the tile of u_c e^{-i k_m.x}, factorised: each thread
// sums its site column over z for kz = 0, 1, 2 (it re-reads the u it wrote);
// the block sums the columns over x for kx = -2..2 per row, then over y per
// mode; one FP64 atomic per value; the block that finishes last (of nblk)
// turns acc into the next coefficients. scr: shared scratch of PT_SCRATCH
// floats that nothing else uses any more; s_tx (cos kx x, -sin kx x) and s_ty
// (e^{i ky y}) are the block's halo-indexed twiddle tables.
constexpr int PT_NV = 15;  // column values: per component sum u, Re/Im sum u e^{-iz}, Re/Im sum u e^{-2iz}
constexpr int PT_NR = SNK * 3 * 3 * TY;  // row sums (kx, c, kz, row), complex
constexpr int PT_SCRATCH = PT_NV * NT + 2 * PT_NR + 2 * FIN_SCRATCH;
static_assert(3 * 3 * 3 * TY <= NT, "one row sum of kx >= 0 per thread");

// this thread's column sums over z of the new u it wrote (planes z0 .. z1-1):
// cs[c][0] = sum u_c, cs[c][1..2] = Re, Im of sum u_c e^{-iz}, cs[c][3..4] of
// sum u_c e^{-2iz}
__device__ __forceinline__ void project_columns(const FastArgs& a, int gxd, int gyd, int z0, int z1, bool act,
                                                float (&cs)[3][5]) {
    const int nx = a.nx, nz = a.nz;
    const unsigned N = (unsigned)a.N, nxy = (unsigned)a.nx * (unsigned)a.ny;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int j = 0; j < 5; ++j) cs[c][j] = 0.f;
    if (act) {
        // planes in batches of PB: all of a batch's loads are in flight together
        constexpr int PB = 8;
        const unsigned col = (unsigned)gyd * (unsigned)nx + (unsigned)gxd;
        for (int zb = z0; zb < z1; zb += PB) {
            float u[PB][3];
            float2 e1[PB], e2[PB];
#pragma unroll
            for (int k = 0; k < PB; ++k) {
                const int z = zb + k;
                if (z < z1) {
                    const unsigned s = (unsigned)z * nxy + col;
#pragma unroll
                    for (int c = 0; c < 3; ++c) u[k][c] = a.maco[(unsigned)(c + 1) * N + s];  // written by this thread
                    int i2 = 2 * z;
                    i2 = i2 >= nz ? i2 - nz : i2;
                    e1[k] = __ldg(a.twz + z);
                    e2[k] = __ldg(a.twz + i2);
                }
            }
#pragma unroll
            for (int k = 0; k < PB; ++k) {
                if (zb + k < z1) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        cs[c][0] += u[k][c];
                        cs[c][1] = fmaf(u[k][c], e1[k].x, cs[c][1]);
                        cs[c][2] = fmaf(-u[k][c], e1[k].y, cs[c][2]);
                        cs[c][3] = fmaf(u[k][c], e2[k].x, cs[c][3]);
                        cs[c][4] = fmaf(-u[k][c], e2[k].y, cs[c][4]);
                    }
                }
            }
        }
    }
}

// the block part of the projection, from every thread's column sums cs
__device__ __forceinline__ void project_tile_sums(const FastArgs& a, float* scr, const float2* s_tx,
                                                  const float2* s_ty, const float (&cs)[3][5], unsigned rep) {
    const int tid = threadIdx.x;
    float* sC = scr;                                    // [PT_NV][NT]
    float2* sR = reinterpret_cast<float2*>(scr + PT_NV * NT);  // [SNK][3][3][TY]
    __syncthreads();  // every warp is past its last use of the scratch region
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int j = 0; j < 5; ++j) sC[(c * 5 + j) * NT + tid] = cs[c][j];
    __syncthreads();
    // row sums over x: thread (kxa, c, kz, row) forms kx = +kxa and -kxa together
    if (tid < 3 * 3 * 3 * TY) {
        const int row = tid % TY, kz = (tid / TY) % 3, c = (tid / (3 * TY)) % 3, kxa = tid / (9 * TY);
        const int vr = c * 5 + (kz == 0 ? 0 : 2 * kz - 1);
        const float* cr = sC + vr * NT + row * TX;
        const float* ci = sC + (vr + 1) * NT + row * TX;  // read only for kz > 0
        const float2* e = s_tx + (kxa + SK) * EX1 + 1;
        const int lane = tid & 31;
        float P = 0.f, Qs = 0.f, R = 0.f, S = 0.f;
#pragma unroll 8
        for (int i = 0; i < TX; ++i) {
            const int xx = (i + lane) & (TX - 1);  // rotated: no bank conflicts
            const float r = cr[xx], im = kz ? ci[xx] : 0.f;
            const float2 t = e[xx];  // (cos, -sin) of kxa x
            P = fmaf(r, t.x, P);
            Qs = fmaf(-im, t.y, Qs);
            R = fmaf(im, t.x, R);
            S = fmaf(-r, t.y, S);
        }
        // (r + i im) e^{-i kxa x} = (P + Qs) + i (R - S); with e^{+i kxa x}: (P - Qs) + i (R + S)
        sR[(((kxa + SK) * 3 + c) * 3 + kz) * TY + row] = make_float2(P + Qs, R - S);
        if (kxa) sR[(((SK - kxa) * 3 + c) * 3 + kz) * TY + row] = make_float2(P - Qs, R + S);
    }
    __syncthreads();
    // per mode and component: sum over rows with e^{-i ky y}, one FP64 atomic each for Re, Im
    for (int t = tid; t < 3 * a.nm; t += NT) {
        const int c = t / a.nm, m = t - c * a.nm;
        const int4 md = __ldg(a.modes + m);
        const float2* r = sR + (((md.x + SK) * 3 + c) * 3 + md.z) * TY;
        const float2* ey = s_ty + (md.y + SK) * EY1 + 1;
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int row = 0; row < TY; ++row) {
            const float2 v = r[row], w = ey[row];  // v e^{-i ky y} = v conj(w)
            re += v.x * w.x + v.y * w.y;
            im += v.y * w.x - v.x * w.y;
        }
        double* dst = a.acc + (size_t)(rep % SP_NREP) * (6 * a.nm) + 2 * (c * a.nm + m);
        atomicAdd(dst, (double)re);
        atomicAdd(dst + 1, (double)im);
    }
}

__device__ __forceinline__ void project_tile(const FastArgs& a, float* scr, const float2* s_tx, const float2* s_ty,
                                             int gxd, int gyd, int z0, int z1, bool act, unsigned rep) {
    float cs[3][5];
    project_columns(a, gxd, gyd, z0, z1, act, cs);
    project_tile_sums(a, scr, s_tx, s_ty, cs, rep);
}

// after all of the block's tiles: the block that finishes last (of nblk) turns
// acc into the next coefficients (scratch as for project_tile)
__device__ __forceinline__ void spectral_block_done(const FastArgs& a, float* scr, unsigned nblk) {
    __threadfence();
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(&a.st->sp_done, 1u) == nblk - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    spectral_finalize(a, reinterpret_cast<double*>(scr + PT_NV * NT + 2 * PT_NR));
    if (threadIdx.x == 0) a.st->sp_done = 0u;
}

// host side shared by the pull (step_fast.cu) and push (step_push.cu) forms
void fill_fast(dl_handle* h, FastArgs& a);
int force_fmode(const dl_handle* h);
void advance(dl_handle* h, int n);
void wall_terms(const dl_handle* h, long long step, float* bot, float* top);

}  // namespace dl
