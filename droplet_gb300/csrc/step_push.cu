// step_push.cu -- the push form of the FP32 step: every site is collided by
// its own thread, with its own record in registers, and streamed by the
// store (f*_i(x) written to x + c_i).
//
// The pull form (step_fast.cu) collides each population at its source from
// the destination's thread, which reads the source's record from shared
// memory once per direction. Here the thread that owns site x loads its 15 f
// and 15 g (its own address: aligned, coalesced), takes their moments, and,
// once the moments of the neighbouring sites are in shared memory, builds its
// record (p0, the phi stencils, the Smagorinsky strain, 1/tau_g) and
// relaxes all 15 directions in registers, pairing each direction with its
// opposite (c.u, c.grad phi and c.F change sign, the even parts are shared).
// The arithmetic is that of program/lbm_drop_xy.f90:421-515 (equilibrium_cal
// and fg_cal, collision at the source) and :517-552 (physics' moments), in
// FP32 and a different order of evaluation.
//
// The moments a kernel takes are those of the populations it loads, i.e. of
// the state before its collision: the reference's physics for the previous
// step. Launch n+1 therefore knows phi, u, p of step n, not of step n+1, and
// two things of step n's streaming are completed when the next launch loads
// the populations ("pending"):
//   * the band force (program/lbm_drop_iht_xy.f90:722-842) depends on u of
//     the step it acts in, which the whole grid computes in this launch; the
//     launch projects it (the last block turns the sums into coefficients)
//     and the next launch adds 3 E_i c_i . F(x - c_i) to every g_i it loads;
//   * the moving-wall reflection (bounce_back_LBM,
//     prototype_program/two-phase/drop8_mpi.f90:642-674) replaces the g that
//     arrive at the wall planes, which the loading thread does.
// A settle launch (SETTLE) completes them in place and writes phi, u, p, the
// phi range and the band coefficients, after which the state is that of the
// pull form. The handle settles before anything reads its fields or
// populations.
//
// Per block: a 32 x 8 tile of columns marching up z. Every plane's moments
// (dphi, u) of the tile and a one-cell ring around it go to a four-slot ring
// in shared memory; with a pending band force, the force of a two-cell ring
// is synthesised per plane into a four-slot ring (Fx, Fy, Fz). One barrier
// per plane. The populations of plane z+1 are loaded while plane z is
// collided: into registers (option "stage" 0), or staged in shared memory one
// plane ahead by per-thread 4-byte asynchronous copies (1) or by two tensor
// copies per plane (TMA, box 32 x 8 x 1 x 15 of the f and g arrays) that
// complete on an mbarrier (2).
//
// Eligible: FP32 storage, viscosity ratio 1 or the fixed-viscosity mode (the
// step's tau_g then needs no phi range of the state it collides), band
// forcing with kc <= 3 or no band forcing.
#include "fast_common.cuh"

#include <cuda.h>  // CUtensorMap and the encoder's enums (the encoder is resolved at run time)

namespace dl {

constexpr int PSL = 4;   // ring slots (moments and band force)
constexpr int FENT = 4;  // band force entry: Fx, Fy, Fz, padding
constexpr int NHALO = 2 * EX1 + 2 * TY;  // 84 positions of the one-cell ring
static_assert(NHALO <= NT, "one halo site per thread at most");
static_assert((PSL & (PSL - 1)) == 0, "ring slots by bit mask");

__device__ __forceinline__ void cp_async4(float* smem_dst, const float* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// a population of the loaded state: read once per step, so it takes no L1 line
// (L1 stays for the kernel's register spill, which it would otherwise evict)
__device__ __forceinline__ float ld_stream(const float* p) {
    float v;
    asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

// ---- tensor copies (TMA) completing on an mbarrier ----
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(b), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b), "r"(bytes) : "memory");
}
// box {32, 8, 1, 15} at (x, y, z, 0) of a 4-d map [15][nz][ny][nx] into dst
__device__ __forceinline__ void tma_load_plane(float* dst, const CUtensorMap* map, unsigned long long* bar, int x,
                                               int y, int z) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(d),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(0), "r"(b)
        : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}
// wait for the phase with the given parity to complete; false once limit_ns
// nanoseconds have passed without it
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned long long limit_ns) {
    const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
    const unsigned long long t0 = global_ns();
    for (;;) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(b), "r"(parity)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

struct PushArgs {
    FastArgs a;
    int pending;           // the loaded populations lack the band force and wall reflection of their streaming
    int walls_load;        // reflect at the wall planes (pending and walls on)
    float wl_bot[5], wl_top[5];  // wall terms of the step whose streaming the load completes
    unsigned long long wait_ns;  // stage 2: limit of a wait for the staged plane (option "wait_ns")
    unsigned extra_tx;           // stage 2: bytes expected beyond the copies' (option "stage_extra_tx", tests
                                 // of the limit: with it no phase completes and every block's wait runs out)
    CUtensorMap tmf, tmg;  // stage 2: maps [15][nz][ny][nx] of the loaded f and g (box 32 x 8 x 1 x 15)
};

// staged populations of the next plane, one column per thread: [2 Q][NT]
constexpr int PB_FLOATS = 2 * Q * NT;
// floats of the staged plane: f and g, or (single phase) g only, at this offset
__host__ __device__ constexpr int pb_floats(bool sp) { return sp ? Q * NT : PB_FLOATS; }
__host__ __device__ constexpr int pb_goff(bool sp) { return sp ? 0 : Q * NT; }

// shared-memory footprint in floats
// (rings and tables, then, stage 1 or 2, the staged plane at a 128-byte
// offset, then, stage 2, its mbarrier and 128 bytes of room to move the plane
// to a 128-byte boundary of the shared window, where tensor copies land)
__host__ __device__ constexpr int push_rings_floats(bool spec, bool sp) {
    return (sp ? 0 : PSL * P1 * 4 + 2 * Q * NHALO) +
           (spec ? PSL * P2 * FENT + 2 * (3 * SNK * EY2 * 2) + 3 * SNK * EY2 * 3 * 2 + SNK * EX2 * 2 +
                       SNK * EY2 * 2 + SNK * EX1 * 2 + SNK * EY1 * 2
                 : 0);
}
__host__ __device__ constexpr int push_stage_offset(bool spec, bool sp) { return (push_rings_floats(spec, sp) + 31) / 32 * 32; }
__host__ __device__ constexpr int push_smem_floats(bool spec, bool sp, int stage = 0) {
    return stage == 0 ? push_rings_floats(spec, sp) : push_stage_offset(spec, sp) + pb_floats(sp) + (stage == 2 ? 36 : 0);
}
static_assert(PSL * P1 * 4 + PSL * P2 * FENT >= PT_SCRATCH, "projection scratch exceeds the rings");

// ring position (1-cell halo coordinates ex, ey in [0, EX1) x [0, EY1)) of the
// thread's halo site h = 0 .. NHALO-1
__device__ __forceinline__ void halo_pos(int h, int& ex, int& ey) {
    if (h < EX1) {
        ex = h;
        ey = 0;
    } else if (h < 2 * EX1) {
        ex = h - EX1;
        ey = EY1 - 1;
    } else if (h < 2 * EX1 + TY) {
        ex = 0;
        ey = 1 + h - 2 * EX1;
    } else {
        ex = EX1 - 1;
        ey = 1 + h - 2 * EX1 - TY;
    }
}

// sum of v[0 .. n-1] as a balanced tree (short dependency chains; the
// order of the additions is fixed by the code, not left to the compiler)
template <int N>
__device__ __forceinline__ float tsum(const float* v) {
    if constexpr (N == 1) return v[0];
    else if constexpr (N == 2) return v[0] + v[1];
    else return tsum<N / 2>(v) + tsum<N - N / 2>(v + N / 2);
}

// packed FP32x2 helpers
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// the moments-ring entry of the stencil neighbour x + c_i of the site at ring index k0
template <int I>
__device__ __forceinline__ float4 nb(const float4* ml, const float4* mc, const float4* mh, int k0) {
    const float4* pl = cz(I) == 0 ? mc : (cz(I) > 0 ? mh : ml);
    return pl[k0 + cy(I) * EX1 + cx(I)];
}
template <int I>
__device__ __forceinline__ float nbx(const float4* ml, const float4* mc, const float4* mh, int k0) {
    const float4* pl = cz(I) == 0 ? mc : (cz(I) > 0 ? mh : ml);
    return reinterpret_cast<const float*>(pl + k0 + cy(I) * EX1 + cx(I))[0];
}

// gradient sums from the differences of the seven opposite pairs:
// d1 = v(+x) - v(-x), d2 (y), d3 (z), d7 .. d10 = v(c) - v(-c) for c = c_7 .. c_10
template <typename T>
__device__ __forceinline__ void pair_grad(T d1, T d2, T d3, T d7, T d8, T d9, T d10, T& gx, T& gy, T& gz);
template <>
__device__ __forceinline__ void pair_grad<float>(float d1, float d2, float d3, float d7, float d8, float d9,
                                                 float d10, float& gx, float& gy, float& gz) {
    const float p = d7 + d8, q = d9 + d10, r = d7 - d8, s = d9 - d10;
    gx = d1 + (r + q);
    gy = d2 + (p - s);
    gz = d3 + (p + s);
}
template <>
__device__ __forceinline__ void pair_grad<float2>(float2 d1, float2 d2, float2 d3, float2 d7, float2 d8, float2 d9,
                                                  float2 d10, float2& gx, float2& gy, float2& gz) {
    const float2 p = add2(d7, d8), q = add2(d9, d10), r = sub2(d7, d8), s = sub2(d9, d10);
    gx = add2(d1, add2(r, q));
    gy = add2(d2, sub2(p, s));
    gz = add2(d3, add2(p, s));
}

// c . v of the four body-diagonal representatives 7 (+,+,+), 8 (-,+,+), 9 (+,-,+), 10 (+,+,-)
__device__ __forceinline__ void diag_dots(float vx, float vy, float vz, float& c7, float& c8, float& c9, float& c10) {
    const float a = vx + vy, b = vx - vy;
    c7 = a + vz;
    c10 = a - vz;
    c9 = b + vz;
    c8 = vz - b;
}

// Record of the site (moments ring, own moments o = dphi, u1, u2, u3, dp), then
// its collision (equilibrium_cal at the site, fg_cal's relaxation and force,
// program/lbm_drop_xy.f90:421-515) and the push of the 30 new populations to
// x + c_i. v[0..14] = df, v[15..29] = dg of the site, deviations of the FP32
// form: df_i = f_i - (H_i phi1 + F_i p0(phi1)), dg_i = g_i - E_i.
template <bool LES, int FMODE, bool SP>
__device__ __forceinline__ void collide_push(const PushArgs& pa, int t, const float* v, const float* o,
                                             const float4* ml, const float4* mc, const float4* mh, int k0,
                                             const unsigned* xs, const unsigned* yr, float mn, float kscale) {
    const FastArgs& a = pa.a;
    const unsigned N = (unsigned)a.N;
    const unsigned nxy = (unsigned)a.nx * (unsigned)a.ny;
    unsigned zo[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) zo[d] = (unsigned)wrap_near(t - 1 + d, a.nz) * nxy;
    float dphi, u1, u2, u3;
    if (SP) {
        dphi = o[0];
        u1 = o[1];
        u2 = o[2];
        u3 = o[3];
    } else {
        const float4 own = mc[k0];  // this site's moments, written to the ring before the barrier
        dphi = own.x;
        u1 = own.y;
        u2 = own.z;
        u3 = own.w;
    }
    const float dp = o[4];
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    if (FMODE == F_ARRAY) {
        const unsigned s = zo[1] + yr[1] + xs[1];
        Fx = __ldg(a.force + s);
        Fy = __ldg(a.force + N + s);
        Fz = __ldg(a.force + 2 * N + s);
    }
    const float S = site_S(dp, u1, u2, u3);  // 3 dp - 1.5 u^2
    float omg, gx = 0.f, gy = 0.f, gz = 0.f, dA = 0.f, gq = 0.f;
    const float phi = __fadd_rn(a.phi1, dphi);
    if (SP) {
        omg = a.omg_sp;
    } else {
        // the 14-neighbour stencils of various_cal (program/lbm_drop_xy.f90:608-633),
        // accumulated pair by pair (x + c, x - c): sum for the Laplacian,
        // difference for the gradients
        float lap, nut = 0.f;
        if (LES) {
            float2 gA[3], gB[3];  // (d phi, d u1), (d u2, d u3) by x_al, unscaled
            float sums[7];
            {
                // pair (x + c, x - c): sum for the Laplacian, difference for the gradients
                float2 dA[7], dB[7];
                auto pair = [&](int k, float4 vp, float4 vm) {
                    sums[k] = vp.x + vm.x;
                    dA[k] = sub2(f2(vp.x, vp.y), f2(vm.x, vm.y));
                    dB[k] = sub2(f2(vp.z, vp.w), f2(vm.z, vm.w));
                };
                pair(0, nb<1>(ml, mc, mh, k0), nb<4>(ml, mc, mh, k0));
                pair(1, nb<2>(ml, mc, mh, k0), nb<5>(ml, mc, mh, k0));
                pair(2, nb<3>(ml, mc, mh, k0), nb<6>(ml, mc, mh, k0));
                pair(3, nb<7>(ml, mc, mh, k0), nb<11>(ml, mc, mh, k0));
                pair(4, nb<8>(ml, mc, mh, k0), nb<12>(ml, mc, mh, k0));
                pair(5, nb<9>(ml, mc, mh, k0), nb<13>(ml, mc, mh, k0));
                pair(6, nb<10>(ml, mc, mh, k0), nb<14>(ml, mc, mh, k0));
                pair_grad<float2>(dA[0], dA[1], dA[2], dA[3], dA[4], dA[5], dA[6], gA[0], gA[1], gA[2]);
                pair_grad<float2>(dB[0], dB[1], dB[2], dB[3], dB[4], dB[5], dB[6], gB[0], gB[1], gB[2]);
            }
            lap = fmaf(-14.f, dphi, tsum<7>(sums));
            gx = gA[0].x * a.inv_grad;
            gy = gA[1].x * a.inv_grad;
            gz = gA[2].x * a.inv_grad;
            // S:S with S = (grad u + grad u^T)/2 of the unscaled sums; du_c/dx_al:
            // u1: gA[al].y, u2: gB[al].x, u3: gB[al].y
            const float sxy = gA[1].y + gB[0].x, sxz = gA[2].y + gB[0].y, syz = gB[2].x + gB[1].y;
            const float ss = gA[0].y * gA[0].y + gB[1].x * gB[1].x + gB[2].y * gB[2].y +
                             0.5f * (sxy * sxy + sxz * sxz + syz * syz);
            const float tt = 2.f * ss * (a.inv_grad * a.inv_grad);
            nut = tt > 0.f ? a.csd * (tt * rsqrtf(tt)) : 0.f;
        } else {
            float g3[3], sums[7], d[7];
            auto pair = [&](int k, float vp, float vm) {
                sums[k] = vp + vm;
                d[k] = vp - vm;
            };
            pair(0, nbx<1>(ml, mc, mh, k0), nbx<4>(ml, mc, mh, k0));
            pair(1, nbx<2>(ml, mc, mh, k0), nbx<5>(ml, mc, mh, k0));
            pair(2, nbx<3>(ml, mc, mh, k0), nbx<6>(ml, mc, mh, k0));
            pair(3, nbx<7>(ml, mc, mh, k0), nbx<11>(ml, mc, mh, k0));
            pair(4, nbx<8>(ml, mc, mh, k0), nbx<12>(ml, mc, mh, k0));
            pair(5, nbx<9>(ml, mc, mh, k0), nbx<13>(ml, mc, mh, k0));
            pair(6, nbx<10>(ml, mc, mh, k0), nbx<14>(ml, mc, mh, k0));
            pair_grad<float>(d[0], d[1], d[2], d[3], d[4], d[5], d[6], g3[0], g3[1], g3[2]);
            lap = fmaf(-14.f, dphi, tsum<7>(sums));
            gx = g3[0] * a.inv_grad;
            gy = g3[1] * a.inv_grad;
            gz = g3[2] * a.inv_grad;
        }
        lap *= a.inv_lap;
        const float gsq = gx * gx + gy * gy + gz * gz;
        gq = 1.5f * gsq;
        dA = site_dp0<false>(a, dphi) - a.kf * phi * lap - a.kf6 * gsq;
        const float nu = (phi - mn) * kscale + a.nu1;
        omg = __fdividef(1.f, 0.5f + 3.f * (nu + nut) * a.inv_ds + a.anu23);  // tau_g >= 0.5, far below 2^126
    }

    // ---- collision, each direction with its opposite, pushed at once ----
    // f: df* = df + wf (dfeq - df), dfeq_i = [i=0] dphi + F_i dA + E_i (3 phi c.u + kf (4.5 (c.gphi)^2 - |c|^2 gq))
    // g: dg* = dg + wg (dgeq - dg) + 3 E_i c.F, dgeq_i = E_i (S + 3 c.u + 4.5 (c.u)^2 + kg (4.5 (c.gphi)^2 - |c|^2 gq))
    // (the relaxation acts on the small non-equilibrium part eq - v, as fg_cal's
    // f - (f - feq)/tau does, not on two large terms of opposite sign)
    const float wf = a.omf, wg = omg;
    float* fo = (float*)a.fo;
    float* go = (float*)a.go;
    // destination index of direction i (x + c_i, wrapped)
    auto dst = [&](int i) -> unsigned { return (unsigned)i * N + zo[1 + cz(i)] + yr[1 + cy(i)] + xs[1 + cx(i)]; };
    // (the lattice constants multiply as exact pairs, mulc: no bias from their rounding)
    if (!SP) fo[dst(0)] = fmaf(wf, (dphi + mulc(dA, Fd(0))) - v[0], v[0]);
    go[dst(0)] = fmaf(wg, mulc(S, Ed(0)) - v[Q], v[Q]);
    // per class (1 axis, 2 diagonal): even parts and odd coefficients of the equilibria
    float Kf[3] = {0.f, 0.f, 0.f}, Bf[3] = {0.f, 0.f, 0.f}, Af[3] = {0.f, 0.f, 0.f}, Kg[3], Ag[3];
#pragma unroll
    for (int c = 1; c <= 2; ++c) {
        const int i = c == 1 ? 1 : 7;
        const float E = Ew(i);
        if (!SP) {
            Kf[c] = mulc(dA, Fd(c)) - E * c2w(i) * a.kf * gq;
            Bf[c] = mulc(phi, 3.0 * Ed(c));
            Af[c] = (4.5f * E) * a.kf;  // 4.5 E_i = 1/2, 1/16: exact
        }
        Kg[c] = mulc(S - c2w(i) * a.kg * gq, Ed(c));
        Ag[c] = 4.5f * E;
    }
    // c . v for the representatives 1, 2, 3 (axes) and 7, 8, 9, 10 (diagonals)
    const float uxy = u1 + u2, uxmy = u1 - u2;
    const float gxy = gx + gy, gxmy = gx - gy;
    const float Fxy = Fx + Fy, Fxmy = Fx - Fy;
    auto dotc = [](int i, float vx, float vy, float vz, float sxy, float dxy) -> float {
        switch (i) {
            case 1: return vx;
            case 2: return vy;
            case 3: return vz;
            case 7: return sxy + vz;
            case 8: return vz - dxy;
            case 9: return dxy + vz;
            default: return sxy - vz;  // 10
        }
    };
    // representative i (c_i) and its opposite j
    auto pairc = [&](int i, int j, int c) {
        const float cu = dotc(i, u1, u2, u3, uxy, uxmy);
        const double e3 = 3.0 * Ed(c);
        const float gd = mulc(cu, e3);  // odd part of geq
        float fF = 0.f;                 // the force term, odd
        if (FMODE == F_ARRAY) fF = mulc(dotc(i, Fx, Fy, Fz, Fxy, Fxmy), e3);
        float ge;
        if (!SP) {
            const float cg = dotc(i, gx, gy, gz, gxy, gxmy);
            const float t = cg * cg;
            const float fe = fmaf(Af[c], t, Kf[c]);
            const float fd = Bf[c] * cu;
            fo[dst(i)] = fmaf(wf, (fe + fd) - v[i], v[i]);
            fo[dst(j)] = fmaf(wf, (fe - fd) - v[j], v[j]);
            ge = fmaf(Ag[c], fmaf(a.kg, t, cu * cu), Kg[c]);
        } else {
            ge = fmaf(Ag[c], cu * cu, Kg[c]);
        }
        go[dst(i)] = fmaf(wg, (ge + gd) - v[Q + i], v[Q + i]) + fF;
        go[dst(j)] = fmaf(wg, (ge - gd) - v[Q + j], v[Q + j]) - fF;
    };
    pairc(1, 4, 1);
    pairc(2, 5, 1);
    pairc(3, 6, 1);
    pairc(7, 11, 2);
    pairc(8, 12, 2);
    pairc(9, 13, 2);
    pairc(10, 14, 2);
}

// block min / max of phi (one atomic per block) and the last block's range of
// the step's loaded state; the reference's rare serial-scan case (the first
// site holds the smallest value while every value exceeds phi1) needs the
// stored field, so it is resolved when the state settles
__device__ __forceinline__ void push_minmax(const FastArgs& a, float bmin, float bmax, bool bad, unsigned nblk) {
    __shared__ float smn[NWARP], smx[NWARP];
    __shared__ int s_bad, s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_bad = 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bmin = fminf(bmin, __shfl_xor_sync(0xffffffffu, bmin, o));
        bmax = fmaxf(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
    }
    __syncthreads();
    if (bad) s_bad = 1;
    if (lane == 0) {
        smn[warp] = bmin;
        smx[warp] = bmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < NWARP; ++w) {
            bmin = fminf(bmin, smn[w]);
            bmax = fmaxf(bmax, smx[w]);
        }
        atomicMin(&a.st->key_min, dbl_key((double)bmin));
        atomicMax(&a.st->key_max, dbl_key((double)bmax));
        if (s_bad) {
            if (atomicExch(&a.st->nan_flag, 1) == 0) a.st->nan_step = a.step;
        }
        __threadfence();
        s_last = (atomicAdd(&a.st->blocks_done, 1u) == nblk - 1);
        if (s_last) {
            __threadfence();
            const long long K0 = atomicAdd((unsigned long long*)&a.st->key_min, 0ull);
            const long long K1 = atomicAdd((unsigned long long*)&a.st->key_max, 0ull);
            const double gmin = key_dbl(K0), gmax = key_dbl(K1);
            a.st->phi_max = gmax > (double)a.phi1 ? gmax : (double)a.phi1;
            a.st->phi_min = gmin < (double)a.phi2 ? gmin : (double)a.phi2;
            a.st->key_min = KEY_POS_INF;
            a.st->key_max = KEY_NEG_INF;
            __threadfence();
            a.st->blocks_done = 0u;
        }
    }
}

// the push-form kernel body. SP: the single-phase step (g only, no stencils).
// SETTLE: no collision; complete the pending part of the loaded state in
// place and write phi, u, p, the phi range and the band coefficients.
// STG 1 and 2: the populations of the next plane arrive in shared memory,
// copied one plane ahead right after the barrier, instead of loaded into
// registers after the collision: by each thread for its own site (4-byte
// asynchronous copies, STG 1), or by one thread for the block (two tensor
// copies completing on an mbarrier, STG 2; full tiles only)
template <bool LES, int FMODE, bool SP, bool SETTLE, int STG = 0>
__device__ __forceinline__ void push_body(const PushArgs& pa, float* smem, int bx, int by, int bz, unsigned nblk) {
    constexpr bool BULK = STG != 0;
    constexpr bool TMA = STG == 2;
    constexpr bool SPEC = FMODE == F_SPECTRAL;
    constexpr bool HALO = !SP && !SETTLE;  // the ring around the tile (stencils)
    constexpr bool NEEDG_HALO = LES;       // halo sites need u (strain) only with LES
    const FastArgs& a = pa.a;
    float4* s_mom = reinterpret_cast<float4*>(smem);              // [PSL][P1] (dphi, u1, u2, u3)
    float* s_h = smem + PSL * P1 * 4;                              // [2 Q][NHALO] halo sites' populations
    float* s_fr = smem + (SP ? 0 : PSL * P1 * 4 + 2 * Q * NHALO);  // [PSL][P2][FENT]
    float2* s_C = reinterpret_cast<float2*>(s_fr + PSL * P2 * FENT);  // [2][3][SNK][EY2]
    float2* s_D = s_C + 2 * 3 * SNK * EY2;                         // [3][SNK][EY2][3]
    float2* s_tx2 = s_D + 3 * SNK * EY2 * 3;                       // [SNK][EX2] (cos, -sin) kx x, x = x0-2+ex
    float2* s_ty2 = s_tx2 + SNK * EX2;                             // [SNK][EY2] e^{i ky y}, y = y0-2+ey
    float2* s_tx1 = s_ty2 + SNK * EY2;                             // [SNK][EX1] projection tables
    float2* s_ty1 = s_tx1 + SNK * EX1;                             // [SNK][EY1]
    float* s_pb = smem + push_stage_offset(SPEC, SP);  // staged plane (BULK): [2 Q][NT], single phase [Q][NT]
    if (TMA) {  // at a 128-byte boundary of the shared window (the room is in the footprint)
        const unsigned off = (unsigned)__cvta_generic_to_shared(s_pb);
        s_pb += ((128u - (off & 127u)) & 127u) / 4u;
    }
    unsigned long long* s_bar = reinterpret_cast<unsigned long long*>(s_pb + pb_floats(SP));  // (TMA)
    float* s_pg = s_pb + pb_goff(SP);  // the staged g

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const unsigned N = (unsigned)a.N;
    const unsigned nxy = (unsigned)nx * (unsigned)ny;
    const int x0 = bx * TX, y0 = by * TY;
    const int z0 = bz * a.lz, z1 = min(z0 + a.lz, nz);
    const bool pend = pa.pending != 0;
    const bool fpend = SPEC && pend;  // band force to add at load

    // own site (wrapped: positions past a partial tile hold the wrapped site)
    const int gxd = x0 + tx, gyd = y0 + ty;
    const bool act = gxd < nx && gyd < ny;
    const unsigned col = (unsigned)pmod(gxd, nx) + (unsigned)nx * (unsigned)pmod(gyd, ny);
    const int kown = (ty + 1) * EX1 + (tx + 1);
    unsigned xs[3], yr[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        xs[d] = (unsigned)pmod(gxd - 1 + d, nx);
        yr[d] = (unsigned)nx * (unsigned)pmod(gyd - 1 + d, ny);
    }
    // halo site of this thread (HALO, tid < NHALO)
    int hex = 0, hey = 0;
    if (HALO && tid < NHALO) halo_pos(tid, hex, hey);
    const bool has_h = HALO && tid < NHALO;
    const unsigned hcol = (unsigned)pmod(x0 - 1 + hex, nx) + (unsigned)nx * (unsigned)pmod(y0 - 1 + hey, ny);
    const int kh = hey * EX1 + hex;

    float mn = a.phi1, mx = a.phi2;
    if (!a.visc_fixed) {
        mn = (float)a.st->phi_min;
        mx = (float)a.st->phi_max;
    }
    const float kscale = a.dnu / (mx - mn);  // zero: eligible only with nu2 = nu1 or the fixed mode

    // ---- band force tables (pending band force) ----
    auto dtable = [&]() {
        for (int t = tid; t < 3 * SNK * EY2 * 3; t += NT) {
            const int kz = t % 3, r = t / 3, yy = r % EY2, r2 = r / EY2, kxi = r2 % SNK, c = r2 / SNK;
            float re = 0.f, im = 0.f;
            const int m1 = a.kx_off[kxi + 1];
            for (int m = a.kx_off[kxi]; m < m1; ++m) {
                const int4 md = __ldg(a.modes + m);
                if (md.z != kz) continue;
                const float2 ey = s_ty2[(md.y + SK) * EY2 + yy];
                const float2 fv = __ldg(a.fh + c * a.nm + m);
                re += fv.x * ey.x - fv.y * ey.y;
                im += fv.x * ey.y + fv.y * ey.x;
            }
            s_D[t] = make_float2(re, im);
        }
    };
    auto ztw = [&](int zr, float2& ez1, float2& ez2) {
        const int zw = wrap_near(zr, nz);
        int i2 = 2 * zw;
        i2 = i2 >= nz ? i2 - nz : i2;
        ez1 = __ldg(a.twz + zw);
        ez2 = __ldg(a.twz + i2);
    };
    // C[c][kx][row] of plane zr into slot zr & 1
    auto ctable = [&](int zr) {
        float2 ez1, ez2;
        ztw(zr, ez1, ez2);
        float2* C = s_C + (zr & 1) * (3 * SNK * EY2);
        for (int t = NT - 1 - tid; t < 3 * SNK * EY2; t += NT) {
            const float2 d0 = s_D[3 * t], d1 = s_D[3 * t + 1], d2 = s_D[3 * t + 2];
            C[t] = make_float2(d0.x + (d1.x * ez1.x - d1.y * ez1.y) + (d2.x * ez2.x - d2.y * ez2.y),
                               d0.y + (d1.x * ez1.y + d1.y * ez1.x) + (d2.x * ez2.y + d2.y * ez2.x));
        }
    };
    // band force of plane zr at every position of the two-cell ring, from slot zr & 1 of C
    auto fsynth = [&](int zr) {
        const float2* C = s_C + (zr & 1) * (3 * SNK * EY2);
        float* dst = s_fr + (size_t)(zr & (PSL - 1)) * (P2 * FENT);
        for (int k = tid; k < P2; k += NT) {
            const int ex = k % EX2, ey = k / EX2;
            float2 acc[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
            for (int kxi = 0; kxi < SNK; ++kxi) {
                const float2 e = s_tx2[kxi * EX2 + ex];
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[c] = __ffma2_rn(C[(c * SNK + kxi) * EY2 + ey], e, acc[c]);
            }
            const float Fx = acc[0].x + acc[0].y, Fy = acc[1].x + acc[1].y, Fz = acc[2].x + acc[2].y;
            reinterpret_cast<float4*>(dst)[k] = make_float4(Fx, Fy, Fz, 0.f);
        }
    };
    // c_i . F from a force-ring entry e (Fx, Fy, Fz), for direction i
    auto cFe = [](const float* e, int i) -> float {
        if (wclass(i) == 1) {
            const int ax = cx(i) != 0 ? 0 : (cy(i) != 0 ? 1 : 2);
            const float v = e[ax];
            return (cx(i) + cy(i) + cz(i)) > 0 ? v : -v;
        }
        const float4 F = *reinterpret_cast<const float4*>(e);
        return cdot3(i, F.x, F.y, F.z);
    };

    // ---- loads and moments ----
    // 15 f and 15 g of the site at column c of plane zp (wrapped)
    auto issue = [&](int zp, unsigned c, float* v, bool withf, bool withg) {
        const unsigned s = (unsigned)wrap_near(zp, nz) * nxy + c;
        if (withf) {
#pragma unroll
            for (int i = 0; i < Q; ++i) v[i] = ld_stream((const float*)a.f + (unsigned)i * N + s);
        }
        if (withg) {
#pragma unroll
            for (int i = 0; i < Q; ++i) v[Q + i] = ld_stream((const float*)a.g + (unsigned)i * N + s);
        }
    };
    // the pending part of the loaded g of the site at ring position (ex, ey) of plane zp:
    // the band force of its sources, then the wall reflection
    auto fslot = [&](int zr) -> const float* { return s_fr + (size_t)(zr & (PSL - 1)) * (P2 * FENT); };
    auto complete = [&](int zp, int ex, int ey, float* g) {
        if (SPEC && fpend) {
            const int k2 = (ey + 1) * EX2 + (ex + 1);
            const float* fl = fslot(zp - 1) + k2 * FENT;  // sources below (c_z = +1)
            const float* fm = fslot(zp) + k2 * FENT;
            const float* fh = fslot(zp + 1) + k2 * FENT;  // sources above (c_z = -1)
#pragma unroll
            for (int i = 1; i < Q; ++i) {
                const float* e = (cz(i) > 0 ? fl : (cz(i) < 0 ? fh : fm)) - (cy(i) * EX2 + cx(i)) * FENT;
                g[i] = fmaf(3.f * Ew(i), cFe(e, i), g[i]);
            }
        }
        if (pa.walls_load) {
            const int zw = wrap_near(zp, nz);
            // bounce_back_LBM, prototype_program/two-phase/drop8_mpi.f90:651-671
            if (zw == 0) {
                g[3] = g[6] - pa.wl_bot[0];
                g[7] = g[11] - pa.wl_bot[1];
                g[8] = g[12] - pa.wl_bot[2];
                g[9] = g[13] - pa.wl_bot[3];
                g[14] = g[10] - pa.wl_bot[4];
            }
            if (zw == nz - 1) {
                g[6] = g[3] - pa.wl_top[0];
                g[10] = g[14] - pa.wl_top[1];
                g[11] = g[7] - pa.wl_top[2];
                g[12] = g[8] - pa.wl_top[3];
                g[13] = g[9] - pa.wl_top[4];
            }
        }
    };
    // moments (physics, program/lbm_drop_xy.f90:541-552) of the deviations
    auto moments = [&](const float* f, const float* g, bool withf, float& dphi, float& u1, float& u2, float& u3,
                       float& dp) {
        dphi = withf ? tsum<Q>(f) : 0.f;
        // opposite pairs: sums for p, differences for u
        const float d1 = g[1] - g[4], d2 = g[2] - g[5], d3 = g[3] - g[6];
        const float d7 = g[7] - g[11], d8 = g[8] - g[12], d9 = g[9] - g[13], d10 = g[10] - g[14];
        pair_grad<float>(d1, d2, d3, d7, d8, d9, d10, u1, u2, u3);
        dp = mulc(tsum<Q>(g), 1.0 / 3.0);
    };

    // ---- staged planes (BULK) ----
    // STG 1: the thread's site of plane zp into its own column of s_pb (4-byte
    // asynchronous copies, coalesced per warp; each thread reads back its own).
    // STG 2: the tile of plane zp, 15 f then 15 g of 256 sites, in the same
    // layout, by two tensor copies; every thread waits for the mbarrier's phase
    // (the copies are issued after a barrier that follows every read of s_pb)
    unsigned tph = 0;       // TMA: parity of the phase the next take waits for
    bool tma_late = false;  // TMA: a wait of this thread ran out (the step reports DL_ERR_TIMEOUT);
                            // thread 0 then issues no more copies and no more waits are made
    auto bulk_issue = [&](int zp) {
        if (!BULK) return;
        if (TMA) {
            if (tid == 0 && !tma_late) {
                const int zw = wrap_near(zp, nz);
                mbar_expect_tx(s_bar, (SP ? 1u : 2u) * Q * NT * (unsigned)sizeof(float) + pa.extra_tx);
                if (!SP) tma_load_plane(s_pb, &pa.tmf, s_bar, x0, y0, zw);
                tma_load_plane(s_pg, &pa.tmg, s_bar, x0, y0, zw);
            }
            return;
        }
        const unsigned s = (unsigned)wrap_near(zp, nz) * nxy + col;
        if (!SP) {
#pragma unroll
            for (int i = 0; i < Q; ++i) cp_async4(s_pb + i * NT + tid, (const float*)a.f + (unsigned)i * N + s);
        }
#pragma unroll
        for (int i = 0; i < Q; ++i) cp_async4(s_pg + i * NT + tid, (const float*)a.g + (unsigned)i * N + s);
        cp_async_commit();
    };
    auto bulk_take = [&](float* v) {
        if (!BULK) return;
        if (TMA) {
            if (!tma_late && !mbar_wait(s_bar, tph, pa.wait_ns)) {
                tma_late = true;
                atomicExch(&a.st->wait_timeout, 1);
            }
            tph ^= 1u;
        } else {
            cp_async_wait_all();
        }
        if (!SP) {
#pragma unroll
            for (int i = 0; i < Q; ++i) v[i] = s_pb[i * NT + tid];
        }
#pragma unroll
        for (int i = 0; i < Q; ++i) v[Q + i] = s_pg[i * NT + tid];
    };

    // ---- prologue: band force tables and planes ----
    if (SPEC) {
        if (fpend) {
            for (int t = tid; t < SNK * EX2; t += NT) {
                const int kxi = t / EX2, ex = t % EX2;
                const float2 e = a.twx[pmod((kxi - SK) * pmod(x0 - 2 + ex, nx), nx)];
                s_tx2[t] = make_float2(e.x, -e.y);
            }
            for (int t = tid; t < SNK * EY2; t += NT) {
                const int kyi = t / EY2, ey = t % EY2;
                s_ty2[t] = a.twy[pmod((kyi - SK) * pmod(y0 - 2 + ey, ny), ny)];
            }
        }
        tile_twiddles(a, s_tx1, s_ty1, x0, y0);
        __syncthreads();
        if (fpend) {
            dtable();
            __syncthreads();
        }
    }
    // band force planes of the prologue. Loading plane p reads F(p-1 .. p+1); the
    // march (HALO) loads z0-1 and z0 here and the first iteration reads
    // F(z0 .. z0+2) and synthesises F(z0+3) from C(z0+3); a settle loads z0 first.
    // Four force slots and two table slots: a plane's table is written one barrier
    // before its synthesis, a slot is rewritten only after its last reader's barrier.
    const int zlo = (HALO ? z0 - 1 : z0);  // first plane loaded
    if (fpend) {
        ctable(zlo - 1);
        ctable(zlo);
        __syncthreads();
        fsynth(zlo - 1);
        fsynth(zlo);
        __syncthreads();
        ctable(zlo + 1);
        ctable(zlo + 2);
        __syncthreads();
        fsynth(zlo + 1);
        if (HALO) fsynth(zlo + 2);
        __syncthreads();
        // march (HALO): F(z0-2 .. z0+1) ready; F(z0+2), F(z0+3) follow the first loads.
        // settle: F(z0-1 .. z0+1) ready, C(z0+2) waits in its slot.
    }
    float bmin = INFINITY, bmax = -INFINITY;
    bool bad = false;
    float cs[3][5];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int j = 0; j < 5; ++j) cs[c][j] = 0.f;

    // the interior site's moments of plane zp: ring entry, range, projection sums, and
    // (SETTLE) the completed g and the fields
    auto own_plane = [&](int zp, float* v, float& dphi, float& u1, float& u2, float& u3, float& dp) {
        complete(zp, tx + 1, ty + 1, v + Q);
        moments(v, v + Q, !SP, dphi, u1, u2, u3, dp);
        if (!SP && !SETTLE) s_mom[(zp & (PSL - 1)) * P1 + kown] = make_float4(dphi, u1, u2, u3);
        const bool inner = zp >= z0 && zp < z1;  // a plane this block owns
        if (act && inner) {
            const float ph = a.phi1 + dphi;
            bmin = fminf(bmin, ph);
            bmax = fmaxf(bmax, ph);
            bad |= !isfinite(dphi + dp + u1 + u2 + u3);
            if (SPEC) {
                float2 e1, e2;
                ztw(zp, e1, e2);
                const float uu[3] = {u1, u2, u3};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    cs[c][0] += uu[c];
                    cs[c][1] = fmaf(uu[c], e1.x, cs[c][1]);
                    cs[c][2] = fmaf(-uu[c], e1.y, cs[c][2]);
                    cs[c][3] = fmaf(uu[c], e2.x, cs[c][3]);
                    cs[c][4] = fmaf(-uu[c], e2.y, cs[c][4]);
                }
            }
            if (SETTLE) {
                const unsigned s = (unsigned)zp * nxy + col;
                if (pend) {
#pragma unroll
                    for (int i = 0; i < Q; ++i) ((float*)a.go)[(unsigned)i * N + s] = v[Q + i];
                }
                a.maco[s] = dphi;
                a.maco[N + s] = u1;
                a.maco[2 * N + s] = u2;
                a.maco[3 * N + s] = u3;
                a.maco[4 * N + s] = dp;
            }
        }
    };
    // the halo site's populations of plane zp into shared memory (asynchronous
    // copies: no registers held while they arrive; each thread reads back its own)
    auto issue_halo = [&](int zp) {
        if (!has_h) return;
        const unsigned s = (unsigned)wrap_near(zp, nz) * nxy + hcol;
#pragma unroll
        for (int i = 0; i < Q; ++i) cp_async4(s_h + i * NHALO + tid, (const float*)a.f + (unsigned)i * N + s);
        if (NEEDG_HALO) {
#pragma unroll
            for (int i = 0; i < Q; ++i)
                cp_async4(s_h + (Q + i) * NHALO + tid, (const float*)a.g + (unsigned)i * N + s);
        }
        cp_async_commit();
    };
    // the halo site's moments of plane zp into the ring, streamed pair by pair
    // from shared memory (band force of the sources, wall reflection, sums)
    auto halo_plane = [&](int zp) {
        if (!has_h) return;
        cp_async_wait_all();
        float hf[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) hf[i] = s_h[i * NHALO + tid];
        const float dphi = tsum<Q>(hf);
        float u1 = 0.f, u2 = 0.f, u3 = 0.f;
        if (NEEDG_HALO) {
            const int zw = wrap_near(zp, nz);
            const bool bot = pa.walls_load && zw == 0, top = pa.walls_load && zw == nz - 1;
            const int k2 = (hey + 1) * EX2 + (hex + 1);
            const float* fl = fslot(zp - 1) + k2 * FENT;
            const float* fm = fslot(zp) + k2 * FENT;
            const float* fh = fslot(zp + 1) + k2 * FENT;
            auto gl = [&](int i) -> float {
                float g = s_h[(Q + i) * NHALO + tid];
                if (SPEC && fpend) {
                    const float* e = (cz(i) > 0 ? fl : (cz(i) < 0 ? fh : fm)) - (cy(i) * EX2 + cx(i)) * FENT;
                    g = fmaf(3.f * Ew(i), cFe(e, i), g);
                }
                return g;
            };
            // the pairs (up, down) across z with their wall-table rows, then the in-plane pairs
            auto zpair = [&](int up, int dn, int kb, int kt, float& gu, float& gd) {
                gu = gl(up);
                gd = gl(dn);
                if (bot) gu = gd - pa.wl_bot[kb];
                if (top) gd = gu - pa.wl_top[kt];
            };
            float gu, gd, d3, d7, d8, d9, d10;
            zpair(3, 6, 0, 0, gu, gd);
            d3 = gu - gd;
            zpair(7, 11, 1, 2, gu, gd);
            d7 = gu - gd;
            zpair(8, 12, 2, 3, gu, gd);
            d8 = gu - gd;
            zpair(9, 13, 3, 4, gu, gd);
            d9 = gu - gd;
            zpair(14, 10, 4, 1, gu, gd);
            d10 = gd - gu;  // c_10 = -c_14
            pair_grad<float>(gl(1) - gl(4), gl(2) - gl(5), d3, d7, d8, d9, d10, u1, u2, u3);
        }
        s_mom[(zp & (PSL - 1)) * P1 + kh] = make_float4(dphi, u1, u2, u3);
    };

    if constexpr (SETTLE) {
        // one plane at a time; before plane zp: F(zp+1) from C(zp+1), then C(zp+2)
        for (int zp = z0; zp < z1; ++zp) {
            if (fpend && zp > z0) {
                __syncthreads();  // the previous plane's readers are done with the slot of F(zp-2)
                fsynth(zp + 1);
                ctable(zp + 2);
                __syncthreads();
            }
            float v[2 * Q];
            issue(zp, col, v, !SP, true);
            float dphi, u1, u2, u3, dp;
            own_plane(zp, v, dphi, u1, u2, u3, dp);
        }
    } else {
        // ---- the march: collide plane t while plane t+1 arrives ----
        float A[2 * Q], B[2 * Q];
        float oA[5], oB[5];  // own moments (dphi, u1, u2, u3, dp) of the planes held in A, B
        if (TMA) {
            if (tid == 0) mbar_init(s_bar, 1);
            __syncthreads();
        }
        // planes zlo (= z0 - 1, moments only) and z0
        if (BULK) {
            bulk_issue(z0 - 1);
            issue_halo(z0 - 1);
            bulk_take(A);
        } else {
            issue(z0 - 1, col, A, !SP, true);
            issue_halo(z0 - 1);
        }
        own_plane(z0 - 1, A, oA[0], oA[1], oA[2], oA[3], oA[4]);
        halo_plane(z0 - 1);
        if (BULK) {
            if (TMA) __syncthreads();  // every thread has read plane z0-1 from s_pb
            bulk_issue(z0);
            issue_halo(z0);
            bulk_take(A);
        } else {
            issue(z0, col, A, !SP, true);
            issue_halo(z0);
        }
        own_plane(z0, A, oA[0], oA[1], oA[2], oA[3], oA[4]);
        halo_plane(z0);
        if (fpend) {
            __syncthreads();  // the loads of z0-1 and z0 have read F(z0-2), F(z0-1) and C(z0), C(z0+1)
            ctable(z0 + 2);
            ctable(z0 + 3);
            __syncthreads();
            fsynth(z0 + 2);
            fsynth(z0 + 3);
            __syncthreads();
        }
        if (BULK) {
            if (TMA && !fpend) __syncthreads();  // every thread has read plane z0 from s_pb
            bulk_issue(z0 + 1);
        } else {
            issue(z0 + 1, col, B, !SP, true);
        }
        issue_halo(z0 + 1);

        // one iteration: moments of plane t+1 (held in nxt), barrier, collide plane t
        // (held in cur), then the loads of plane t+2 into cur
        auto iteration = [&](int t, float* cur, float* nxt, float* ocur, float* onxt) {
            bulk_take(nxt);
            own_plane(t + 1, nxt, onxt[0], onxt[1], onxt[2], onxt[3], onxt[4]);
            halo_plane(t + 1);
            // the table of plane t+4, for this iteration's synthesis after the barrier
            if (fpend) ctable(t + 4);
            __syncthreads();
            // the next planes' populations: in flight during this plane's collision
            if (t + 2 <= z1) {
                bulk_issue(t + 2);
                issue_halo(t + 2);
            }
            // the force of plane t+4, read from iteration t+2 on (after the next barrier)
            if (fpend && t + 4 <= z1 + 1) fsynth(t + 4);
            if (act) {
                const float4* mc = s_mom + (t & (PSL - 1)) * P1;
                const float4* ml = s_mom + ((t - 1) & (PSL - 1)) * P1;
                const float4* mh = s_mom + ((t + 1) & (PSL - 1)) * P1;
                collide_push<LES, FMODE, SP>(pa, t, cur, ocur, ml, mc, mh, kown, xs, yr, mn, kscale);
            }
            if (!BULK && t + 2 <= z1) issue(t + 2, col, cur, !SP, true);
        };
        int t = z0;
        for (; t + 1 < z1; t += 2) {
            iteration(t, A, B, oA, oB);
            iteration(t + 1, B, A, oB, oA);
        }
        if (t < z1) iteration(t, A, B, oA, oB);
    }

    if constexpr (SPEC) {
        project_tile_sums(a, smem, s_tx1, s_ty1, cs, bx + 3 * by + 5 * bz);
        spectral_block_done(a, smem, nblk);
    }
    if constexpr (SETTLE) {
        minmax_block_and_finalize<float>(a.st, (double)bmin, (double)bmax, a.maco, a.phi1, a.N, (double)a.phi1,
                                         (double)a.phi2, bad, a.step, nblk);
    } else {
        push_minmax(a, bmin, bmax, bad, nblk);
    }
    if (TMA && tid == 0 && tma_late) {
        // copies issued before the wait ran out may still be in flight: keep the
        // block, and with it its shared memory, a millisecond longer
        const unsigned long long t0 = global_ns();
        while (global_ns() - t0 < 1000000ull) __nanosleep(10000);
    }
}

template <bool LES, int FMODE, int STG>
__global__ void __launch_bounds__(NT, 2) step_push(const __grid_constant__ PushArgs pa) {
    extern __shared__ __align__(128) float smem[];
    push_body<LES, FMODE, false, false, STG>(pa, smem, blockIdx.x, blockIdx.y, blockIdx.z,
                                             gridDim.x * gridDim.y * gridDim.z);
}

template <int FMODE, int STG>
__global__ void __launch_bounds__(NT, 2) step_push_sp(const __grid_constant__ PushArgs pa) {
    extern __shared__ __align__(128) float smem[];
    push_body<false, FMODE, true, false, STG>(pa, smem, blockIdx.x, blockIdx.y, blockIdx.z,
                                              gridDim.x * gridDim.y * gridDim.z);
}

// an ensemble's push steps as ONE persistent launch: work items (member, tile
// x, tile y, z chunk), largest members first, taken one at a time from a
// counter (zeroed before the launch) by whichever block is free, so that the
// items' uneven lengths even out; each member's last block (of
// nblk_of[member]) finalises its phi range and band coefficients. Up to
// PUSH_CMAX members read their arguments from a constant-memory table (copied
// there before each launch: the same access path as kernel parameters);
// larger ensembles copy them into shared memory per work item.
constexpr int PUSH_CMAX = 64;
__constant__ PushArgs c_members[PUSH_CMAX];

// the next work item of the block (uniform across it)
__device__ __forceinline__ int next_item(unsigned* counter) {
    __shared__ int s_w;
    __syncthreads();  // the previous item's readers of s_w and of the rings are done
    if (threadIdx.x == 0) s_w = (int)atomicAdd(counter, 1u);
    __syncthreads();
    return s_w;
}

template <bool LES, int FMODE>
__global__ void __launch_bounds__(NT, 2) step_push_batched_c(const int4* __restrict__ items, int nitems,
                                                             const unsigned* __restrict__ nblk_of,
                                                             unsigned* counter) {
    extern __shared__ __align__(128) float smem[];
    for (int w = next_item(counter); w < nitems; w = next_item(counter)) {
        const int4 it = items[w];
        push_body<LES, FMODE, false, false, 0>(c_members[it.x], smem, it.y, it.z, it.w, nblk_of[it.x]);
    }
}

template <bool LES, int FMODE>
__global__ void __launch_bounds__(NT, 2) step_push_batched(const PushArgs* __restrict__ table,
                                                           const int4* __restrict__ items, int nitems,
                                                           const unsigned* __restrict__ nblk_of, unsigned* counter) {
    extern __shared__ __align__(128) float smem[];
    __shared__ PushArgs s_pa;
    for (int w = next_item(counter); w < nitems; w = next_item(counter)) {
        const int4 it = items[w];
        const int* src = reinterpret_cast<const int*>(table + it.x);
        int* dst = reinterpret_cast<int*>(&s_pa);
        for (int t = threadIdx.x; t < (int)(sizeof(PushArgs) / sizeof(int)); t += blockDim.x) dst[t] = src[t];
        __syncthreads();
        push_body<LES, FMODE, false, false, 0>(s_pa, smem, it.y, it.z, it.w, nblk_of[it.x]);
    }
}

template <int FMODE, bool SP>
__global__ void __launch_bounds__(NT, 2) settle_push(const PushArgs pa) {
    extern __shared__ __align__(128) float smem[];
    push_body<false, FMODE, SP, true>(pa, smem, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x * gridDim.y * gridDim.z);
}

// ---- host side ------------------------------------------------------------------
bool push_eligible(const dl_handle* h) {
    if (h->form != DL_FORM_FP32 || !h->push) return false;
    const dl_params& P = h->P;
    // tau_g must not depend on the phi range of the state being collided
    if (!(P.nu2 == P.nu1 || P.visc_mode == DL_VISC_FIXED)) return false;
    // kc > 3: the force arrays are computed from the current u by separate launches
    if (h->force_mode == DL_FORCE_SPECTRAL && h->fsp.nm == 0) return false;
    return true;
}

// arguments of a push step (settle = false) or of the settle of the current state
static void push_args(dl_handle* h, PushArgs& pa, bool settle) {
    memset(&pa, 0, sizeof(pa));
    FastArgs& a = pa.a;
    fill_fast(h, a);
    const int c = h->cur, n = 1 - c;
    a.f = h->fs[c];
    a.g = h->gs[c];
    a.fo = settle ? nullptr : h->fs[n];
    a.go = settle ? h->gs[c] : h->gs[n];
    a.maco = settle ? h->mac32[c] : nullptr;
    a.mac = nullptr;
    a.fh = h->fsp.d_fh[h->fsp.par];
    a.fh_next = h->fsp.d_fh[1 - h->fsp.par];
    a.step = settle ? h->step : h->step + 1;
    pa.pending = h->pushed ? 1 : 0;
    pa.walls_load = (h->pushed && h->P.walls) ? 1 : 0;
    // the load completes the streaming of step h->step
    wall_terms(h, h->step, pa.wl_bot, pa.wl_top);
}

template <typename K>
static int configure_smem(dl_handle* h, K kernel, size_t bytes, bool* done) {
    const int dev = h->device & 63;
    if (!done[dev]) {
        DL_CUDA(h, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        done[dev] = true;
    }
    return DL_OK;
}

static dim3 push_grid(const dl_handle* h, int lz) {
    return dim3((h->nx + TX - 1) / TX, (h->ny + TY - 1) / TY, (h->nz + lz - 1) / lz);
}

// ---- option "stage" 2: tensor maps of the population buffers ----
// f and g of each of the two buffers as 4-d FP32 tensors [15][nz][ny][nx]
// (x innermost), box 32 x 8 x 1 x 15: one copy brings a tile's plane of all
// 15 directions. The encoder is the driver's, resolved at run time (no link
// against the driver library); the maps are made once per handle.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

bool push_tma_eligible(const dl_handle* h) { return h->nx % TX == 0 && h->ny % TY == 0; }

static int make_tmaps(dl_handle* h) {
    if (h->push_tmap_ok) return DL_OK;
    if (!push_tma_eligible(h)) return set_error(h, DL_ERR_UNSUPPORTED, "stage 2 needs nx %% %d == 0 and ny %% %d == 0", TX, TY);
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return set_error(h, DL_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const EncodeTiledFn encode = reinterpret_cast<EncodeTiledFn>(fn);
    const cuuint64_t dims[4] = {(cuuint64_t)h->nx, (cuuint64_t)h->ny, (cuuint64_t)h->nz, (cuuint64_t)Q};
    const cuuint64_t strides[3] = {(cuuint64_t)h->nx * 4, (cuuint64_t)h->nx * h->ny * 4, (cuuint64_t)h->N * 4};
    const cuuint32_t box[4] = {TX, TY, 1, Q};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    void* bufs[4] = {h->fs[0], h->fs[1], h->gs[0], h->gs[1]};
    static_assert(sizeof(CUtensorMap) == sizeof(h->push_tmap[0]), "tensor map size");
    for (int k = 0; k < 4; ++k) {
        if (!bufs[k]) continue;  // the single-phase step has no f
        CUtensorMap m;
        const CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, bufs[k], dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return set_error(h, DL_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        memcpy(h->push_tmap[k], &m, sizeof(m));
    }
    h->push_tmap_ok = 1;
    return DL_OK;
}

template <bool LES, int FMODE, int STG>
static int launch_push_t(dl_handle* h, const PushArgs& pa) {
    static bool done[64] = {false};
    const size_t sm = sizeof(float) * (size_t)push_smem_floats(FMODE == F_SPECTRAL, false, STG);
    int rc = configure_smem(h, step_push<LES, FMODE, STG>, sm, done);
    if (rc != DL_OK) return rc;
    DL_LAUNCH(h, true, (step_push<LES, FMODE, STG><<<push_grid(h, pa.a.lz), NT, sm, h->stream>>>(pa)));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}
template <bool LES, int FMODE>
static int launch_push(dl_handle* h, const PushArgs& pa) {
    return h->push_bulk == 2   ? launch_push_t<LES, FMODE, 2>(h, pa)
           : h->push_bulk == 1 ? launch_push_t<LES, FMODE, 1>(h, pa)
                               : launch_push_t<LES, FMODE, 0>(h, pa);
}

template <int FMODE, int STG>
static int launch_push_sp_t(dl_handle* h, const PushArgs& pa) {
    static bool done[64] = {false};
    const size_t sm = sizeof(float) * (size_t)push_smem_floats(FMODE == F_SPECTRAL, true, STG);
    int rc = configure_smem(h, step_push_sp<FMODE, STG>, sm, done);
    if (rc != DL_OK) return rc;
    DL_LAUNCH(h, true, (step_push_sp<FMODE, STG><<<push_grid(h, pa.a.lz), NT, sm, h->stream>>>(pa)));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}
template <int FMODE>
static int launch_push_sp(dl_handle* h, const PushArgs& pa) {
    return h->push_bulk == 2   ? launch_push_sp_t<FMODE, 2>(h, pa)
           : h->push_bulk == 1 ? launch_push_sp_t<FMODE, 1>(h, pa)
                               : launch_push_sp_t<FMODE, 0>(h, pa);
}

template <int FMODE, bool SP>
static int launch_settle(dl_handle* h, const PushArgs& pa) {
    static bool done[64] = {false};
    const size_t sm = sizeof(float) * (size_t)push_smem_floats(FMODE == F_SPECTRAL, SP);
    int rc = configure_smem(h, settle_push<FMODE, SP>, sm, done);
    if (rc != DL_OK) return rc;
    DL_LAUNCH(h, false, (settle_push<FMODE, SP><<<push_grid(h, pa.a.lz), NT, sm, h->stream>>>(pa)));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int push_step(dl_handle* h) {
    PushArgs pa;
    push_args(h, pa, false);
    if (h->push_bulk == 2) {
        const int rc = make_tmaps(h);
        if (rc != DL_OK) return rc;
        pa.wait_ns = (unsigned long long)h->push_wait_ns;
        pa.extra_tx = (unsigned)h->push_extra_tx;
        memcpy(&pa.tmf, h->push_tmap[h->cur], sizeof(pa.tmf));
        memcpy(&pa.tmg, h->push_tmap[2 + h->cur], sizeof(pa.tmg));
    }
    const int fmode = force_fmode(h);
    int rc;
    if (h->single) {
        rc = fmode == F_SPECTRAL ? launch_push_sp<F_SPECTRAL>(h, pa)
           : fmode == F_ARRAY    ? launch_push_sp<F_ARRAY>(h, pa)
                                 : launch_push_sp<F_NONE>(h, pa);
    } else if (h->P.les) {
        rc = fmode == F_SPECTRAL ? launch_push<true, F_SPECTRAL>(h, pa)
           : fmode == F_ARRAY    ? launch_push<true, F_ARRAY>(h, pa)
                                 : launch_push<true, F_NONE>(h, pa);
    } else {
        rc = fmode == F_SPECTRAL ? launch_push<false, F_SPECTRAL>(h, pa)
           : fmode == F_ARRAY    ? launch_push<false, F_ARRAY>(h, pa)
                                 : launch_push<false, F_NONE>(h, pa);
    }
    if (rc != DL_OK) return rc;
    advance(h, 1);  // the launch wrote the next band coefficients (from the u it loaded)
    h->pushed = 1;
    h->fsp.dirty = 0;
    return DL_OK;
}

// ---- ensembles: the members' push steps as one persistent launch ----
size_t push_args_bytes() { return sizeof(PushArgs); }

// arguments of the push step k (0 or 1) steps after the handle's current
// state, which must be a push step's (pending); for the tables a captured pair
// of steps replays
void push_args_at(dl_handle* h, int k, void* out) {
    PushArgs pa;
    memset(&pa, 0, sizeof(pa));
    FastArgs& a = pa.a;
    fill_fast(h, a);
    const int c = h->cur ^ (k & 1), n = 1 - c;
    a.f = h->fs[c];
    a.g = h->gs[c];
    a.fo = h->fs[n];
    a.go = h->gs[n];
    a.maco = nullptr;
    a.mac = nullptr;
    const int par = force_fmode(h) == F_SPECTRAL ? (h->fsp.par ^ (k & 1)) : h->fsp.par;
    a.fh = h->fsp.d_fh[par];
    a.fh_next = h->fsp.d_fh[1 - par];
    a.step = h->step + 1 + k;
    pa.pending = 1;
    pa.walls_load = h->P.walls ? 1 : 0;
    wall_terms(h, h->step + k, pa.wl_bot, pa.wl_top);
    memcpy(out, &pa, sizeof(pa));
}

template <bool LES, int FMODE>
static int launch_push_batched_t(dl_handle* h0, const void* table, int nm, const int4* items, int nitems,
                                 const unsigned* nblk, unsigned* counter, int grid, cudaStream_t s) {
    const size_t sm = sizeof(float) * (size_t)push_smem_floats(FMODE == F_SPECTRAL, false);
    DL_CUDA(h0, cudaMemsetAsync(counter, 0, sizeof(unsigned), s));
    if (nm <= PUSH_CMAX) {
        static bool done[64] = {false};
        int rc = configure_smem(h0, step_push_batched_c<LES, FMODE>, sm, done);
        if (rc != DL_OK) return rc;
        DL_CUDA(h0, cudaMemcpyToSymbolAsync(c_members, table, (size_t)nm * sizeof(PushArgs), 0,
                                            cudaMemcpyDeviceToDevice, s));
        step_push_batched_c<LES, FMODE><<<grid, NT, sm, s>>>(items, nitems, nblk, counter);
    } else {
        static bool done[64] = {false};
        int rc = configure_smem(h0, step_push_batched<LES, FMODE>, sm, done);
        if (rc != DL_OK) return rc;
        step_push_batched<LES, FMODE><<<grid, NT, sm, s>>>(static_cast<const PushArgs*>(table), items, nitems, nblk,
                                                           counter);
    }
    DL_CUDA(h0, cudaGetLastError());
    return DL_OK;
}

int launch_push_batched(dl_handle* h0, const void* table, int nm, const int4* items, int nitems,
                        const unsigned* nblk, unsigned* counter, int grid, cudaStream_t s) {
    const int fmode = force_fmode(h0);
#define DL_PB(L, F) launch_push_batched_t<L, F>(h0, table, nm, items, nitems, nblk, counter, grid, s)
    if (h0->P.les)
        return fmode == F_SPECTRAL ? DL_PB(true, F_SPECTRAL) : fmode == F_ARRAY ? DL_PB(true, F_ARRAY) : DL_PB(true, F_NONE);
    return fmode == F_SPECTRAL ? DL_PB(false, F_SPECTRAL) : fmode == F_ARRAY ? DL_PB(false, F_ARRAY) : DL_PB(false, F_NONE);
#undef DL_PB
}

int fast_settle(dl_handle* h) {
    if (!h->pushed) return DL_OK;
    PushArgs pa;
    push_args(h, pa, true);
    const bool spec = force_fmode(h) == F_SPECTRAL;
    int rc;
    if (h->single) rc = spec ? launch_settle<F_SPECTRAL, true>(h, pa) : launch_settle<F_NONE, true>(h, pa);
    else rc = spec ? launch_settle<F_SPECTRAL, false>(h, pa) : launch_settle<F_NONE, false>(h, pa);
    if (rc != DL_OK) return rc;
    if (spec) h->fsp.par = 1 - h->fsp.par;  // coefficients of the settled u
    h->pushed = 0;
    return DL_OK;
}

}  // namespace dl
