// step_fast.cu -- the reduced-precision forms as ONE fused kernel per time step.
//
// Arithmetic is FP32. Populations are stored
//   FP32 form: as deviations from the bulk equilibrium at phi = phi1, p = 1/3,
//              u = 0:  df_i = f_i - (H_i phi1 + F_i p0(phi1)),  dg_i = g_i - E_i;
//   FP16 form: as FP16 residuals against the local part of the equilibrium,
//              r_i = df_i - (H_i dphi + F_i dp0(phi) + 3 E_i phi c_i.u),
//              s_i = dg_i - E_i (3 dp + 3 c_i.u + 4.5 (c_i.u)^2 - 1.5 u^2),
//              rebuilt from the FP32 moments of the same site when read.
// The macroscopic fields are FP32: dphi = phi - phi1, u, dp = p - 1/3.
//
// One launch does all of program/lbm_drop_xy.f90:830-840 for a block's tile
// (what the reference spreads over various_cal, gphi_cal, equilibrium_cal,
// fg_cal and physics, with feq/geq, gradients and fnext materialised):
//   * the block owns a 32 x 8 column tile and marches up a range of z planes;
//   * phi (and u for the Smagorinsky strain) are staged plane by plane in
//     shared memory with a two-cell halo, by asynchronous copies issued one
//     iteration ahead (4-plane ring);
//   * for every site of the tile plus a one-cell halo a "record" is built
//     once: dphi, u, the feq bracket dA, S = 3dp - 1.5u^2, 1/tau_g (with the
//     eddy viscosity), grad(phi) and the body force (4-plane ring); the
//     records of plane z+2 are built in the same barrier interval as the pull
//     of plane z, one barrier per plane;
//   * each thread pulls its 15 f and 15 g from x - c_i (prefetched into
//     registers before the record stage), collides each at its source from
//     that source's record (feq_i, geq_i built on the fly, never stored),
//     applies the moving-wall bounce-back, takes the moments, stores
//     populations and fields, and reduces phi min/max; the last block turns
//     the reduction into the next step's tau_g range.
// Body force (FMODE):
//   F_NONE     no force;
//   F_ARRAY    Fx, Fy, Fz read from HBM at the record sites (static force, or
//              the spectral force for kc > 3 computed by separate launches);
//   F_SPECTRAL the band forcing of program/lbm_drop_iht_xy.f90:722-842 done
//              inside the step: the force at each record site is synthesised
//              from the band coefficients through a per-plane table in shared
//              memory; after its march each block projects the new u of its
//              own tile on the band modes (column sums over z for kz = 0..2,
//              then rows over x and modes over y in shared memory, one set of
//              FP64 atomics per block; option "projection" = 0: a launch of
//              its own, sp_project_fast), and the last block turns the sums
//              into the next step's coefficients. No force array touches HBM.
#include "fast_common.cuh"

namespace dl {

// ---- the fused step kernel ---------------------------------------------------
// Per z plane one barrier: the staging ring and the record ring have four
// slots; the records of plane z+2 are built in the same barrier interval as
// the pull of plane z. Records are float4 groups:
//   q0 = (dphi, u1, u2, u3), q1 = (gx, gy, gz, dA), q2 = (S, 1/tau_g, dp0 (FP16) or 1.5|grad phi|^2 (FP32), Fx),
//   q3 = (Fy, Fz) (with a force only).
constexpr int NSLOT = 4;

__device__ __forceinline__ void cp_async4(float* smem_dst, const float* gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// bulk prefetch of [p, p + bytes) into L2 (16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// shared-memory footprint (floats) of the fused kernel; the single-phase step
// stages nothing and keeps records q0, q2 (and q3)
__host__ __device__ constexpr int fused_smem_floats(bool les, bool spec, bool force, bool sp = false) {
    return (sp ? 0 : NSLOT * P2 * (les ? 4 : 1)) + NSLOT * P1 * ((sp ? 8 : 12) + (force ? 2 : 0)) +
           (spec ? 2 * (2 * 3 * SNK * EY1) + 2 * (SNK * EX1 + SNK * EY1) + 2 * (3 * 3 * SNK * EY1) : 0);
}
// the in-step projection's scratch lies below the spectral tables in every form
static_assert(NSLOT * P1 * 10 >= PT_SCRATCH, "projection scratch exceeds the record ring");

// the thread's (at most two) record positions: pass A = its own column
// (rows 0..7, cols 0..31), pass B = rows 8..9 and columns 32..33
struct RecPos {
    int k, ex, ey;
    bool has;
};
__device__ __forceinline__ RecPos rec_pos(int tid, int j) {
    RecPos r;
    if (j == 0) {
        r.ex = tid % TX;
        r.ey = tid / TX;
        r.has = true;
    } else if (tid < 2 * TX) {
        r.ex = tid % TX;
        r.ey = TY + tid / TX;
        r.has = true;
    } else if (tid < 2 * TX + 2 * EY1) {
        r.ex = TX + (tid - 2 * TX) % 2;
        r.ey = (tid - 2 * TX) / 2;
        r.has = true;
    } else {
        r.ex = r.ey = 0;
        r.has = false;
    }
    r.k = r.ey * EX1 + r.ex;
    return r;
}

// SP: the single-phase step (g only; no staging, no phi stencils).
// PIPE (SP only): the next plane's pulls are issued before this plane's
// collision, so two planes of loads are in flight per thread.
template <typename ST, bool RES, bool LES, int FMODE, bool SP = false, bool PIPE = false>
__device__ __forceinline__ void fused_body(const FastArgs& a, float* smem, int bx, int by, int z0, int z1, float& bmin,
                                           float& bmax, bool& bad) {
    constexpr bool FORCE = FMODE != F_NONE;
    constexpr bool SPEC = FMODE == F_SPECTRAL;
    constexpr int NSTG = LES ? 4 : 1;                    // staged fields: phi (+ u1, u2, u3)
    float* s_stg = smem;                                 // [NSLOT][NSTG][P2] (none for SP)
    float4* s_q0 = (float4*)(s_stg + (SP ? 0 : NSLOT * NSTG * P2));  // [NSLOT][P1]
    float4* s_q1 = s_q0 + NSLOT * P1;                    // (not used by SP)
    float4* s_q2 = s_q1 + (SP ? 0 : NSLOT * P1);
    float2* s_q3 = (float2*)(s_q2 + NSLOT * P1);         // [NSLOT][P1] (FORCE)
    float2* s_C = s_q3 + (FORCE ? NSLOT * P1 : 0);       // [2][3][SNK][EY1] (SPEC)
    float2* s_tx = s_C + 2 * 3 * SNK * EY1;              // [SNK][EX1] (cos kx x, -sin kx x)
    float2* s_ty = s_tx + SNK * EX1;                     // [SNK][EY1] e^{i ky y}
    float2* s_D = s_ty + SNK * EY1;                      // [3][SNK][EY1][3] z-free part of C, by kz
    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const unsigned N = (unsigned)a.N;
    const unsigned nxy = (unsigned)nx * (unsigned)ny;
    const int x0 = bx * TX, y0 = by * TY;
    float mn, mx;
    if (a.visc_fixed) {
        mn = a.phi1;
        mx = a.phi2;
    } else {
        mn = (float)a.st->phi_min;
        mx = (float)a.st->phi_max;
    }
    const float kscale = a.dnu / (mx - mn);  // nu = (phi - mn) kscale + nu1
    // ---- per-thread wrapped offsets (computed once) ----
    unsigned soff[2];  // staging positions k = tid, tid + NT (P2 = 432 < 2 NT)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int k = tid + j * NT;
        const int ex = k % EX2, ey = k / EX2;
        soff[j] = k < P2 ? (unsigned)pmod(x0 - 2 + ex, nx) + (unsigned)nx * (unsigned)pmod(y0 - 2 + ey, ny) : 0u;
    }
    unsigned roff[2];  // record positions
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const RecPos rp = rec_pos(tid, j);
        roff[j] = rp.has ? (unsigned)pmod(x0 - 1 + rp.ex, nx) + (unsigned)nx * (unsigned)pmod(y0 - 1 + rp.ey, ny) : 0u;
    }
    const int gxd = x0 + tx, gyd = y0 + ty;
    const bool act = gxd < nx && gyd < ny;
    unsigned xs[3], yr[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        xs[d] = (unsigned)pmod(gxd - 1 + d, nx);
        yr[d] = (unsigned)nx * (unsigned)pmod(gyd - 1 + d, ny);
    }
    if (SPEC) tile_twiddles(a, s_tx, s_ty, x0, y0);
    // record-site values read from HBM one plane ahead (p, and u without LES)
    float pf_dp[2], pf_u[2][3];
    auto prefetch = [&](int zr) {
        const unsigned zo = (unsigned)wrap_near(zr, nz) * nxy;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const bool has = j == 0 || tid < 2 * TX + 2 * EY1;
            if (!has) continue;
            const unsigned s = zo + roff[j];
            pf_dp[j] = __ldg(a.mac + 4 * N + s);
            if (!LES) {
                pf_u[j][0] = __ldg(a.mac + N + s);
                pf_u[j][1] = __ldg(a.mac + 2 * N + s);
                pf_u[j][2] = __ldg(a.mac + 3 * N + s);
            }
        }
    };

    auto stage = [&](int zz) {  // asynchronous copy of plane zz (wrapped) into its slot
        if constexpr (SP) return;
        const int slot = (zz + NSLOT) % NSLOT;
        const unsigned zo = (unsigned)wrap_near(zz, nz) * nxy;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int k = tid + j * NT;
            if (k >= P2) continue;
            const unsigned s = zo + soff[j];
            if (LES) {  // pairs (phi - phi1, u1) then (u2, u3)
                float* dst = s_stg + slot * NSTG * P2 + 2 * k;
                cp_async4(dst, a.mac + s);
                cp_async4(dst + 1, a.mac + N + s);
                cp_async4(dst + 2 * P2, a.mac + 2 * N + s);
                cp_async4(dst + 2 * P2 + 1, a.mac + 3 * N + s);
            } else {
                cp_async4(s_stg + slot * NSTG * P2 + k, a.mac + s);
            }
        }
        cp_async_commit();
    };

    // force synthesis table of plane zr: C[c][kx][row] = sum over the modes with
    // this kx of w f_hat e^{i (ky y + kz z)} = sum_kz D[c][kx][row][kz] e^{i kz z},
    // D built once per block (dtable), C per plane from the two z twiddles
    auto dtable = [&]() {
        for (int t = tid; t < 3 * SNK * EY1 * 3; t += NT) {
            const int kz = t % 3, r = t / 3, yy = r % EY1, r2 = r / EY1, kxi = r2 % SNK, c = r2 / SNK;
            float re = 0.f, im = 0.f;
            const int m1 = a.kx_off[kxi + 1];
            for (int m = a.kx_off[kxi]; m < m1; ++m) {
                const int4 md = __ldg(a.modes + m);
                if (md.z != kz) continue;
                const float2 ey = s_ty[(md.y + SK) * EY1 + yy];
                const float2 fv = __ldg(a.fh + c * a.nm + m);
                re += fv.x * ey.x - fv.y * ey.y;
                im += fv.x * ey.y + fv.y * ey.x;
            }
            s_D[t] = make_float2(re, im);
        }
    };
    auto ctable = [&](int zr, float2 ez1, float2 ez2) {
        float2* C = s_C + ((zr + 2) & 1) * (3 * SNK * EY1);
        // the last warps take the table: the first ones carry the halo records
        for (int t = NT - 1 - tid; t < 3 * SNK * EY1; t += NT) {
            const float2 d0 = s_D[3 * t], d1 = s_D[3 * t + 1], d2 = s_D[3 * t + 2];
            C[t] = make_float2(d0.x + (d1.x * ez1.x - d1.y * ez1.y) + (d2.x * ez2.x - d2.y * ez2.y),
                               d0.y + (d1.x * ez1.y + d1.y * ez1.x) + (d2.x * ez2.y + d2.y * ez2.x));
        }
    };
    // e^{i z} and e^{2 i z} of plane zr
    auto ztw = [&](int zr, float2& ez1, float2& ez2) {
        const int zw = wrap_near(zr, nz);
        int i2 = 2 * zw;
        i2 = i2 >= nz ? i2 - nz : i2;
        ez1 = __ldg(a.twz + zw);
        ez2 = __ldg(a.twz + i2);
    };

    auto records = [&](int zr) {
        const int sc = (zr + NSLOT) % NSLOT, sm1 = (zr + NSLOT - 1) % NSLOT, sp1 = (zr + 1) % NSLOT;
        const float2* C = s_C + ((zr + 2) & 1) * (3 * SNK * EY1);
        const float* stc = s_stg + sc * NSTG * P2;
        const float* stm = s_stg + sm1 * NSTG * P2;
        const float* stp = s_stg + sp1 * NSTG * P2;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const RecPos rp = rec_pos(tid, j);
            if (!rp.has) continue;
            float F[3] = {0.f, 0.f, 0.f};
            if (FMODE == F_ARRAY) {
                const unsigned s = (unsigned)wrap_near(zr, nz) * nxy + roff[j];
                F[0] = __ldg(a.force + s);
                F[1] = __ldg(a.force + N + s);
                F[2] = __ldg(a.force + 2 * N + s);
            } else if (SPEC) {
                // F_c = sum_kx Re(C e^{i kx x}): one FFMA2 per term, the two lanes added at the end
                float2 acc[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
                for (int kxi = 0; kxi < SNK; ++kxi) {
                    const float2 e = s_tx[kxi * EX1 + rp.ex];
#pragma unroll
                    for (int c = 0; c < 3; ++c) acc[c] = __ffma2_rn(C[(c * SNK + kxi) * EY1 + rp.ey], e, acc[c]);
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) F[c] = acc[c].x + acc[c].y;
            }
            const int o = sc * P1 + rp.k;
            if constexpr (SP) {
                const float u1 = pf_u[j][0], u2 = pf_u[j][1], u3 = pf_u[j][2];
                s_q0[o] = make_float4(0.f, u1, u2, u3);
                s_q2[o] = make_float4(site_S(pf_dp[j], u1, u2, u3), a.omg_sp, 0.f, F[0]);
                if (FORCE) s_q3[o] = make_float2(F[1], F[2]);
                continue;
            }
            const int c2 = (rp.ey + 1) * EX2 + (rp.ex + 1);
            Rec r;
            if constexpr (LES) {
                float2 pa[Q], pb[Q];
#pragma unroll
                for (int i = 1; i < Q; ++i) {
                    const float* st = cz(i) == 0 ? stc : (cz(i) > 0 ? stp : stm);
                    const int q = c2 + cy(i) * EX2 + cx(i);
                    pa[i] = reinterpret_cast<const float2*>(st)[q];
                    pb[i] = reinterpret_cast<const float2*>(st + 2 * P2)[q];
                }
                const float2 ca = reinterpret_cast<const float2*>(stc)[c2];
                const float2 cb = reinterpret_cast<const float2*>(stc + 2 * P2)[c2];
                r = make_record_les2<RES>(a, ca.x, pa, pb, ca.y, cb.x, cb.y, pf_dp[j], mn, kscale);
            } else {
                float v[Q];
#pragma unroll
                for (int i = 1; i < Q; ++i) {
                    const float* st = cz(i) == 0 ? stc : (cz(i) > 0 ? stp : stm);
                    v[i] = st[c2 + cy(i) * EX2 + cx(i)];
                }
                r = make_record<false, RES>(a, stc[c2], v, nullptr, pf_u[j][0], pf_u[j][1], pf_u[j][2], pf_dp[j], mn,
                                       kscale);
            }
            s_q0[o] = make_float4(r.dphi, r.u1, r.u2, r.u3);
            s_q1[o] = make_float4(r.gx, r.gy, r.gz, r.dA);
            s_q2[o] = make_float4(r.S, r.omg, RES ? r.dp0 : 1.5f * r.gsq, F[0]);
            if (FORCE) s_q3[o] = make_float2(F[1], F[2]);
        }
    };

    // L2 prefetch of the rows the pulls of plane zp read: per population array
    // and direction, the TY source rows y0-c_y.. at plane zp-c_z, columns
    // x0-1 .. x0+TX (one bulk prefetch per row, clipped to the row and array)
    auto pull_prefetch = [&](int zp) {
        constexpr int NARR = SP ? 1 : 2;
        constexpr unsigned ES = sizeof(ST);
        const int xa = max(x0 - 1, 0), xb = min(x0 + TX + 1, nx);
        for (int t = tid; t < NARR * Q * TY; t += NT) {
            const int r = t % TY, q = t / TY, i = q % Q;
            const bool isg = SP || q >= Q;
            const char* base = (const char*)(isg ? a.g : a.f);
            const size_t arr_end = (size_t)Q * N * ES;
            const size_t row = (size_t)i * N + (size_t)wrap_near(zp - cz(i), nz) * nxy +
                               (size_t)nx * (unsigned)wrap_near(y0 + r - cy(i), ny);
            size_t b0 = (row + (size_t)xa) * ES, b1 = (row + (size_t)xb) * ES;
            b0 &= ~(size_t)15;
            b1 = (b1 + 15) & ~(size_t)15;
            if (b1 > (arr_end & ~(size_t)15)) b1 = arr_end & ~(size_t)15;
            if (b1 > b0) prefetch_l2(base + b0, (unsigned)(b1 - b0));
        }
    };

    // L2 prefetch of the tile's new u rows of planes z0 .. zl-1 (written
    // planes ago, since evicted) for the in-step projection after the march
    auto u_prefetch = [&](int zl) {
        const int xr = min(TX, nx - x0);
        const size_t end = ((size_t)5 * N * sizeof(float)) & ~(size_t)15;
        for (int t = tid; t < 3 * TY * (zl - z0); t += NT) {
            const int r = t % TY, c = (t / TY) % 3, zz = z0 + t / (3 * TY);
            if (y0 + r >= ny) continue;
            const size_t o = (size_t)(c + 1) * N + (size_t)zz * nxy + (size_t)(y0 + r) * nx + x0;
            const size_t b0 = (o * sizeof(float)) & ~(size_t)15;
            size_t b1 = ((o + xr) * sizeof(float) + 15) & ~(size_t)15;
            if (b1 > end) b1 = end;
            if (b1 > b0) prefetch_l2((const char*)a.maco + b0, (unsigned)(b1 - b0));
        }
    };

    // ---- prologue: records of planes z0-1, z0, z0+1 ----
    // Records of plane zr need the staged planes zr-1..zr+1; the chunk needs
    // records z0-1..z1, so planes z0-2..z1+1 are staged. Plane zz is staged
    // right after the barrier that retires the last reader of its slot, half an
    // iteration before its first use.
    stage(z0 - 2);
    stage(z0 - 1);
    stage(z0);
    stage(z0 + 1);
    prefetch(z0 - 1);
    if (SPEC) {
        __syncthreads();  // s_ty, s_tx
        dtable();
        __syncthreads();  // s_D
        float2 e1, e2;
        ztw(z0 - 1, e1, e2);
        ctable(z0 - 1, e1, e2);
        ztw(z0, e1, e2);
        ctable(z0, e1, e2);
    }
    cp_async_wait_all();
    __syncthreads();
    records(z0 - 1);
    prefetch(z0);
    records(z0);
    prefetch(z0 + 1);
    __syncthreads();
    stage(z0 + 2);
    if (SPEC) {
        float2 e1, e2;
        ztw(z0 + 1, e1, e2);
        ctable(z0 + 1, e1, e2);
    }
    cp_async_wait_all();
    __syncthreads();
    if (z0 + 3 <= z1 + 1) stage(z0 + 3);  // slot of z0-1, last read by records(z0)
    records(z0 + 1);
    if (z0 + 2 <= z1) prefetch(z0 + 2);

    // g pulled from x - c_i at plane zp (the PIPE register stage)
    auto pull_g = [&](int zp, float* v) {
        unsigned zq[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) zq[d] = (unsigned)wrap_near(zp - 1 + d, nz) * nxy;
#pragma unroll
        for (int i = 0; i < Q; ++i) v[i] = Pop<ST>::ld(a.g, (unsigned)i * N + zq[1 - cz(i)] + yr[1 - cy(i)] + xs[1 - cx(i)]);
    };
    float gnx[Q];
    if constexpr (PIPE) {
        if (act) pull_g(z0, gnx);
    }

    for (int z = z0; z < z1; ++z) {
        float2 tz1, tz2;  // twiddles of plane z+2 (their latency hides behind the pulls)
        if (SPEC) ztw(z + 2, tz1, tz2);
        // populations of the destination plane, pulled from x - c_i
        unsigned zo[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) zo[d] = (unsigned)wrap_near(z - 1 + d, nz) * nxy;
        float fin[Q], gin[Q];
        if constexpr (PIPE) {
#pragma unroll
            for (int i = 0; i < Q; ++i) gin[i] = gnx[i];
        } else if (act) {
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const unsigned src = zo[1 - cz(i)] + yr[1 - cy(i)] + xs[1 - cx(i)];
                if constexpr (!SP) fin[i] = Pop<ST>::ld(a.f, (unsigned)i * N + src);
                gin[i] = Pop<ST>::ld(a.g, (unsigned)i * N + src);
            }
        }
        if (SPEC && z + 2 <= z1) ctable(z + 2, tz1, tz2);
        cp_async_wait_all();  // plane z+3
        __syncthreads();
        if (z + 4 <= z1 + 1) stage(z + 4);  // slot of plane z, last read by records(z+1)
        if constexpr (PIPE) {
            if (act && z + 1 < z1) pull_g(z + 1, gnx);
        }
        if (a.l2_prefetch && z + 1 < z1) pull_prefetch(z + 1);
        if (SPEC && a.proj_in_step && z == z1 - 1) u_prefetch(z);
        if (z + 2 <= z1) records(z + 2);
        if (z + 3 <= z1) prefetch(z + 3);
        if (act) {
            float fo[Q], go[Q];
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const int o = ((z - cz(i) + NSLOT) % NSLOT) * P1 + (ty + 1 - cy(i)) * EX1 + (tx + 1 - cx(i));
                if constexpr (SP) {
                    const float4 q0 = s_q0[o], q2 = s_q2[o];
                    float Fy = 0.f, Fz = 0.f;
                    if (FORCE) {
                        const float2 q3 = s_q3[o];
                        Fy = q3.x;
                        Fz = q3.y;
                    }
                    go[i] = collide_g<RES, FORCE>(i, q2.x, q2.y, q0.y, q0.z, q0.w, q2.w, Fy, Fz, gin[i]);
                    fo[i] = 0.f;
                    continue;
                }
                const float4 q0 = s_q0[o], q1 = s_q1[o], q2 = s_q2[o];
                Rec r;
                r.dphi = q0.x;
                r.u1 = q0.y;
                r.u2 = q0.z;
                r.u3 = q0.w;
                r.gx = q1.x;
                r.gy = q1.y;
                r.gz = q1.z;
                r.dA = q1.w;
                r.S = q2.x;
                r.omg = q2.y;
                if (RES) {
                    r.dp0 = q2.z;
                    r.gsq = r.gx * r.gx + r.gy * r.gy + r.gz * r.gz;
                } else {
                    r.gq = q2.z;
                }
                if (FORCE) {
                    const float2 q3 = s_q3[o];
                    r.Fx = q2.w;
                    r.Fy = q3.x;
                    r.Fz = q3.y;
                } else {
                    r.Fx = r.Fy = r.Fz = 0.f;
                }
                collide_dir<RES, FORCE>(a, i, r, fin[i], gin[i], fo[i], go[i]);
            }
            if (a.walls) {
                // bounce_back_LBM, prototype_program/two-phase/drop8_mpi.f90:651-671
                if (z == 0) {
                    go[3] = go[6] - a.wall_bot[0];
                    go[7] = go[11] - a.wall_bot[1];
                    go[8] = go[12] - a.wall_bot[2];
                    go[9] = go[13] - a.wall_bot[3];
                    go[14] = go[10] - a.wall_bot[4];
                }
                if (z == nz - 1) {
                    go[6] = go[3] - a.wall_top[0];
                    go[10] = go[14] - a.wall_top[1];
                    go[11] = go[7] - a.wall_top[2];
                    go[12] = go[8] - a.wall_top[3];
                    go[13] = go[9] - a.wall_top[4];
                }
            }
            // moments (physics, program/lbm_drop_xy.f90:541-552)
            float dphin = 0.f, dpn = 0.f, u1n = 0.f, u2n = 0.f, u3n = 0.f;
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                if constexpr (!SP) dphin += fo[i];
                dpn += go[i];
                if (cx(i) == 1) u1n += go[i];
                else if (cx(i) == -1) u1n -= go[i];
                if (cy(i) == 1) u2n += go[i];
                else if (cy(i) == -1) u2n -= go[i];
                if (cz(i) == 1) u3n += go[i];
                else if (cz(i) == -1) u3n -= go[i];
            }
            dpn = mulc(dpn, 1.0 / 3.0);  // exact 1/3: no bias in p from step to step
            const unsigned d = zo[1] + yr[1] + xs[1];
            if (RES) {
                const float phin = __fadd_rn(a.phi1, dphin);
                const float dp0n = site_dp0<RES>(a, dphin);
                const float Sn = site_S(dpn, u1n, u2n, u3n);
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    const float cu = (i == 0) ? 0.f : cdot3(i, u1n, u2n, u3n);
                    if constexpr (!SP) Pop<ST>::st(a.fo, (unsigned)i * N + d, fo[i] - fbar(i, dphin, phin, dp0n, cu));
                    Pop<ST>::st(a.go, (unsigned)i * N + d, go[i] - gbar(i, Sn, cu));
                }
            } else {
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    if constexpr (!SP) Pop<ST>::st(a.fo, (unsigned)i * N + d, fo[i]);
                    Pop<ST>::st(a.go, (unsigned)i * N + d, go[i]);
                }
            }
            a.maco[d] = dphin;
            a.maco[N + d] = u1n;
            a.maco[2 * N + d] = u2n;
            a.maco[3 * N + d] = u3n;
            a.maco[4 * N + d] = dpn;
            const float phin_f = a.phi1 + dphin;
            bmin = fminf(bmin, phin_f);  // fminf ignores NaN
            bmax = fmaxf(bmax, phin_f);
            bad |= !isfinite(dphin + dpn + u1n + u2n + u3n);  // a NaN or infinity in any term reaches the sum
        }
    }
}

// block (bx, by, bz) marches planes bz lz .. bz lz + lz - 1 of its tile, projects
// the new u of its tile (band forcing), then the block-count finalisations
template <typename ST, bool RES, bool LES, int FMODE, bool SP, bool PIPE = false>
__device__ __forceinline__ void fused_grid(const FastArgs& a, float* smem) {
    float bmin = INFINITY, bmax = -INFINITY;
    bool bad = false;
    const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
    const int z0 = blockIdx.z * a.lz, z1 = min(z0 + a.lz, a.nz);
    fused_body<ST, RES, LES, FMODE, SP, PIPE>(a, smem, blockIdx.x, blockIdx.y, z0, z1, bmin, bmax, bad);
    if constexpr (FMODE == F_SPECTRAL) {
        if (a.proj_in_step) {
            // the tile's twiddle tables follow the staging and record rings (the layout of fused_body)
            const float2* s_tx =
                reinterpret_cast<const float2*>(smem + fused_smem_floats(LES, false, true, SP)) + 2 * 3 * SNK * EY1;
            const int gxd = blockIdx.x * TX + (threadIdx.x % TX), gyd = blockIdx.y * TY + threadIdx.x / TX;
            project_tile(a, smem, s_tx, s_tx + SNK * EX1, gxd, gyd, z0, z1, gxd < a.nx && gyd < a.ny,
                         blockIdx.x + 3 * blockIdx.y + 5 * blockIdx.z);
            spectral_block_done(a, smem, nblk);
        }
    }
    minmax_block_and_finalize<float>(a.st, (double)bmin, (double)bmax, a.maco, a.phi1, a.N, (double)a.phi1,
                                     (double)a.phi2, bad, a.step, nblk);
}

// the single-phase step: a third of the two-phase shared memory, three blocks per SM
template <typename ST, bool RES, int FMODE>
__global__ void __launch_bounds__(NT, 3) step_fused_sp(const FastArgs a) {
    extern __shared__ float smem[];
    fused_grid<ST, RES, false, FMODE, true>(a, smem);
}

// the same with the next plane's pulls in registers: two blocks per SM
template <typename ST, bool RES, int FMODE>
__global__ void __launch_bounds__(NT, 2) step_fused_sp_pipe(const FastArgs a) {
    extern __shared__ float smem[];
    fused_grid<ST, RES, false, FMODE, true, true>(a, smem);
}

template <typename ST, bool RES, bool LES, int FMODE, bool SP = false>
__global__ void __launch_bounds__(NT, 2) step_fused(const FastArgs a) {
    extern __shared__ float smem[];
    fused_grid<ST, RES, LES, FMODE, SP>(a, smem);
}

// ---- band projection of the new u (F_SPECTRAL) ---------------------------------------
// acc[c][m] += sum over sites of u_c e^{-i k_m.x}: one warp per (y, z) row,
// lanes over x with the x twiddles, a transposed warp sum of the row's 15
// values, then each lane owns two band modes and applies e^{-i (ky y + kz z)};
// block sum and one FP64 atomic per value; the block that finishes last turns
// acc into the next coefficients.
constexpr int PROJ_NT = 256;
constexpr int SNV = 2 * SK + 1;  // values of a row per component: sum u_c, then Re, Im of k = 1..SK
constexpr int NRV = 16;          // the 3 SNV values padded to 16 for the lane transpose
static_assert(3 * SNV <= NRV, "row values exceed the lane transpose");

// sum of v[0..15] over the warp, transposed: each exchange halves the values a
// lane holds; afterwards lanes 2j and 2j+1 hold the total of value j
__device__ __forceinline__ float warp_transpose_sum16(float (&v)[NRV], int lane) {
#pragma unroll
    for (int h = NRV / 2, o = 16; h >= 1; h >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            const float send = up ? v[j] : v[j + h];
            const float keep = up ? v[j + h] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// k y reduced into [0, n) for |k| <= SK
__device__ __forceinline__ int wrap_k(int ky, int n) {
#pragma unroll
    for (int s = 0; s < SK; ++s) {
        ky = ky < 0 ? ky + n : ky;
        ky = ky >= n ? ky - n : ky;
    }
    return ky;
}

// rows first, first + stride, ... below nrows, one per warp iteration
__device__ void project_rows(const FastArgs& a, int first, int stride, int nrows, unsigned nblk) {
    const int tid = threadIdx.x, lane = tid & 31;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long long N = a.N;
    const float* u[3] = {a.maco + N, a.maco + 2 * N, a.maco + 3 * N};
    // the lane's two modes (absent modes: k = 0, never accumulated)
    int kx[2], ky[2], kz[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int m = lane + 32 * j;
        const int4 md = m < a.nm ? __ldg(a.modes + m) : make_int4(0, 0, 0, 0);
        kx[j] = md.x;
        ky[j] = md.y;
        kz[j] = md.z;
    }
    float pacc[2][3][2];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) pacc[j][c][0] = pacc[j][c][1] = 0.f;
    const int dz = stride / ny, dy = stride - dz * ny;
    int z = first / ny, y = first - z * ny;
    for (int row = first; row < nrows; row += stride) {
        const long long base = (long long)row * nx;
        float v[NRV];
#pragma unroll
        for (int t = 0; t < NRV; ++t) v[t] = 0.f;
#pragma unroll 4
        for (int x = lane; x < nx; x += 32) {
            float uv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) uv[c] = u[c][base + x];
#pragma unroll
            for (int c = 0; c < 3; ++c) v[c * SNV] += uv[c];
#pragma unroll
            for (int k = 1; k <= SK; ++k) {
                int ix = k * x;
#pragma unroll
                for (int s = 1; s < k; ++s) ix = ix >= nx ? ix - nx : ix;
                const float2 e = a.twx[ix];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v[c * SNV + 2 * k - 1] = fmaf(uv[c], e.x, v[c * SNV + 2 * k - 1]);
                    v[c * SNV + 2 * k] = fmaf(-uv[c], e.y, v[c * SNV + 2 * k]);
                }
            }
        }
        const float tot = warp_transpose_sum16(v, lane);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int ak = kx[j] < 0 ? -kx[j] : kx[j];
            const float2 ey = a.twy[wrap_k(ky[j] * y, ny)], ez = a.twz[wrap_k(kz[j] * z, nz)];
            const float pr = ey.x * ez.x - ey.y * ez.y;
            const float pi = -(ey.x * ez.y + ey.y * ez.x);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float xr = __shfl_sync(0xffffffffu, tot, 2 * (c * SNV + (ak ? 2 * ak - 1 : 0)));
                float xi = __shfl_sync(0xffffffffu, tot, 2 * (c * SNV + 2 * ak));
                xi = ak ? (kx[j] < 0 ? -xi : xi) : 0.f;
                pacc[j][c][0] += xr * pr - xi * pi;
                pacc[j][c][1] += xr * pi + xi * pr;
            }
        }
        y += dy;
        z += dz;
        if (y >= ny) {
            y -= ny;
            z += 1;
        }
    }
    const int warp = tid >> 5;
    __shared__ float red[PROJ_NT / 32][3][SMAXM][2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int m = lane + 32 * j;
        if (m < a.nm)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                red[warp][c][m][0] = pacc[j][c][0];
                red[warp][c][m][1] = pacc[j][c][1];
            }
    }
    __syncthreads();
    for (int t = tid; t < 3 * a.nm * 2; t += PROJ_NT) {
        const int part = t & 1, cm = t >> 1, c = cm / a.nm, m = cm % a.nm;
        float s = 0.f;
        for (int w = 0; w < PROJ_NT / 32; ++w) s += red[w][c][m][part];
        atomicAdd(a.acc + (size_t)(blockIdx.x % SP_NREP) * (6 * a.nm) + 2 * (c * a.nm + m) + part, (double)s);
    }
    __threadfence();
    __shared__ int s_last;
    __syncthreads();
    if (tid == 0) {
        const unsigned t = atomicAdd(&a.st->sp_done, 1u);
        s_last = (t == nblk - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    __shared__ double fin[FIN_SCRATCH];
    spectral_finalize(a, fin);
    if (tid == 0) a.st->sp_done = 0u;
}

// rows dealt to the grid's warps in turn, so that every SM gets the same share
__global__ void __launch_bounds__(PROJ_NT, 4) sp_project_fast(const FastArgs a) {
    constexpr int W = PROJ_NT / 32;
    project_rows(a, blockIdx.x * W + (threadIdx.x >> 5), gridDim.x * W, a.ny * a.nz, gridDim.x);
}

// ---- initial populations f = feq, g = geq at every site (ini :244-251) -------
template <typename ST, bool RES>
__global__ void __launch_bounds__(256) init_fast(const FastArgs a) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    const long long N = a.N;
    const long long t = s / a.nx;
    const int x = (int)(s - t * a.nx);
    const int z = (int)(t / a.ny);
    const int y = (int)(t - (long long)z * a.ny);
    float v[Q];
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const long long nb = wrapi(x + cx(i), a.nx) +
                             (long long)a.nx * (wrapi(y + cy(i), a.ny) + (long long)a.ny * wrapi(z + cz(i), a.nz));
        v[i] = a.mac[nb];
    }
    const float u1 = a.mac[N + s], u2 = a.mac[2 * N + s], u3 = a.mac[3 * N + s], dp = a.mac[4 * N + s];
    const Rec r = make_record<false, RES>(a, a.mac[s], v, nullptr, u1, u2, u3, dp, a.phi1, a.dnu / (a.phi2 - a.phi1));
    const float phi = __fadd_rn(a.phi1, r.dphi);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const float cu = (i == 0) ? 0.f : cdot3(i, u1, u2, u3);
        const float cg = (i == 0) ? 0.f : cdot3(i, r.gx, r.gy, r.gz);
        const float cGc = 4.5f * cg * cg - 1.5f * c2w(i) * r.gsq;
        const float E = Ew(i);
        const float dfeq = (i == 0 ? r.dphi : 0.f) + Fw(i) * r.dA + E * (3.f * phi * cu + a.kf * cGc);
        const float dgeq = E * (r.S + cu * (3.f + 4.5f * cu) + a.kg * cGc);
        if (RES) {
            if (a.fo) Pop<ST>::st(a.fo, i * N + s, dfeq - fbar(i, r.dphi, phi, r.dp0, cu));
            Pop<ST>::st(a.go, i * N + s, dgeq - gbar(i, r.S, cu));
        } else {
            if (a.fo) Pop<ST>::st(a.fo, i * N + s, dfeq);
            Pop<ST>::st(a.go, i * N + s, dgeq);
        }
    }
}

// ---- host <-> device conversions -------------------------------------------
// doubles [5][N] (phi, u1, u2, u3, p) -> float deviations
__global__ void fields_to_fast(const double* __restrict__ d, float* __restrict__ m, long long N, double phi1) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= N) return;
    m[s] = (float)(d[s] - phi1);
    m[N + s] = (float)d[N + s];
    m[2 * N + s] = (float)d[2 * N + s];
    m[3 * N + s] = (float)d[3 * N + s];
    m[4 * N + s] = (float)(d[4 * N + s] - 1.0 / 3.0);
}

__global__ void fast_to_fields(const float* __restrict__ m, double* __restrict__ d, long long N, double phi1) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= N) return;
    d[s] = phi1 + (double)m[s];
    d[N + s] = (double)m[N + s];
    d[2 * N + s] = (double)m[2 * N + s];
    d[3 * N + s] = (double)m[3 * N + s];
    d[4 * N + s] = 1.0 / 3.0 + (double)m[4 * N + s];
}

// stored populations -> full f, g as doubles, direction fastest
template <typename ST, bool RES>
__global__ void pops_to_host(const FastArgs a, double* __restrict__ fa, double* __restrict__ ga) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    const long long N = a.N;
    const float dphi = a.mac[s], u1 = a.mac[N + s], u2 = a.mac[2 * N + s], u3 = a.mac[3 * N + s];
    const float dp = a.mac[4 * N + s];
    const float phi = __fadd_rn(a.phi1, dphi);
    const float dp0 = site_dp0<RES>(a, dphi);
    const float S = site_S(dp, u1, u2, u3);
    const double E[3] = {2.0 / 9.0, 1.0 / 9.0, 1.0 / 72.0};
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        double fv = a.f ? (double)Pop<ST>::ld(a.f, i * N + s) : 0.0;
        double gv = (double)Pop<ST>::ld(a.g, i * N + s);
        if (RES) {
            const float cu = (i == 0) ? 0.f : cdot3(i, u1, u2, u3);
            fv += (double)fbar(i, dphi, phi, dp0, cu);
            gv += (double)gbar(i, S, cu);
        }
        fa[s * Q + i] = a.f ? fv + (double)a.fref[i] : 0.0;  // single phase: no f
        ga[s * Q + i] = gv + E[wclass(i)];
    }
}

// full f, g (direction fastest, doubles) -> moments and stored populations
template <typename ST, bool RES>
__global__ void pops_from_host(const FastArgs a, const double* __restrict__ fa, const double* __restrict__ ga) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    const long long N = a.N;
    const double E[3] = {2.0 / 9.0, 1.0 / 9.0, 1.0 / 72.0};
    double ph = 0.0, pp = 0.0, m1 = 0.0, m2 = 0.0, m3 = 0.0;
    float df[Q], dg[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const double fv = fa[s * Q + i], gv = ga[s * Q + i];
        ph += fv;
        pp += gv / 3.0;
        m1 += cx(i) * gv;
        m2 += cy(i) * gv;
        m3 += cz(i) * gv;
        df[i] = (float)(fv - (double)a.fref[i]);
        dg[i] = (float)(gv - E[wclass(i)]);
    }
    const float dphi = a.fo ? (float)(ph - (double)a.phi1) : 0.f;  // single phase: phi = phi1
    const float u1 = (float)m1, u2 = (float)m2, u3 = (float)m3, dp = (float)(pp - 1.0 / 3.0);
    a.maco[s] = dphi;
    a.maco[N + s] = u1;
    a.maco[2 * N + s] = u2;
    a.maco[3 * N + s] = u3;
    a.maco[4 * N + s] = dp;
    const float phi = __fadd_rn(a.phi1, dphi);
    const float dp0 = site_dp0<RES>(a, dphi);
    const float S = site_S(dp, u1, u2, u3);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        float fv = df[i], gv = dg[i];
        if (RES) {
            const float cu = (i == 0) ? 0.f : cdot3(i, u1, u2, u3);
            fv -= fbar(i, dphi, phi, dp0, cu);
            gv -= gbar(i, S, cu);
        }
        if (a.fo) Pop<ST>::st(a.fo, i * N + s, fv);
        Pop<ST>::st(a.go, i * N + s, gv);
    }
}

// band coefficients of the current u from the separable DFT stages
// (u_hat = uh[c][kx][ky][kz], already / N): E, coefficient and fh for the
// in-kernel synthesis; one block
__global__ void sp_fhat_from_uh(const double* __restrict__ uh, int K, const int4* __restrict__ modes, int nm,
                                double half_eps, float2* __restrict__ fh, DevState* st) {
    __shared__ double s_e[8];
    __shared__ double s_coef;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int NK = 2 * K + 1;
    double e = 0.0;
    for (int m = tid; m < nm; m += blockDim.x) {
        const int4 md = modes[m];
        double s = 0.0;
        for (int c = 0; c < 3; ++c) {
            const double* v = uh + 2 * ((((long long)c * NK + (md.x + K)) * NK + (md.y + K)) * (K + 1) + md.z);
            s += v[0] * v[0] + v[1] * v[1];
        }
        e += 0.5 * (double)md.w * s;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if (lane == 0) s_e[warp] = e;
    __syncthreads();
    if (tid == 0) {
        double E = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) E += s_e[w];
        s_coef = half_eps / E;
        st->sp_energy = E;
        st->sp_coef = s_coef;
    }
    __syncthreads();
    for (int t = tid; t < 3 * nm; t += blockDim.x) {
        const int c = t / nm, m = t % nm;
        const int4 md = modes[m];
        const double* v = uh + 2 * ((((long long)c * NK + (md.x + K)) * NK + (md.y + K)) * (K + 1) + md.z);
        const double k = s_coef * (double)md.w;
        fh[t] = make_float2((float)(k * v[0]), (float)(k * v[1]));
    }
}

// ---- host side ---------------------------------------------------------------------
template <bool RES, bool LES, int FMODE, bool SP = false>
static size_t smem_bytes() {
    return sizeof(float) * (size_t)fused_smem_floats(LES, FMODE == F_SPECTRAL, FMODE != F_NONE, SP);
}

void fill_fast(dl_handle* h, FastArgs& a) {
    const dl_params& P = h->P;
    memset(&a, 0, sizeof(a));
    a.nx = h->nx;
    a.ny = h->ny;
    a.nz = h->nz;
    a.lz = h->lz > 0 ? h->lz : std::min(h->nz, DL_DEFAULT_LZ);
    a.l2_prefetch = h->l2_prefetch;
    a.proj_in_step = h->proj_in_step;

    a.N = (long long)h->N;
    a.st = h->d_state;
    a.phi1 = (float)P.phi1;
    a.phi2 = (float)P.phi2;
    a.omf = (float)(1.0 / P.tauf);
    a.kf = (float)P.kappaf;
    a.kf6 = (float)(P.kappaf / 6.0);
    a.kg = (float)P.kappag;
    a.T = (float)P.T;
    a.a = (float)P.a;
    a.b = (float)P.b;
    a.omb1 = (float)(1.0 - P.b * P.phi1);
    a.nu1 = (float)P.nu1;
    a.dnu = (float)(P.nu2 - P.nu1);
    a.csd = (float)(P.Cs * P.Cs * P.delta * P.delta);
    a.anu23 = (float)((2.0 / 3.0) * P.Anu);
    a.inv_ds = (float)(1.0 / P.ds);
    a.omg_sp = 1.f / (0.5f + 3.f * a.nu1 * a.inv_ds + a.anu23);
    a.inv_lap = (float)(1.0 / (5.0 * P.ds * P.ds));
    a.inv_grad = (float)(1.0 / (10.0 * P.ds));
    const double p0ref = P.phi1 * P.T / (1.0 - P.b * P.phi1) - P.a * P.phi1 * P.phi1;
    for (int i = 0; i < Q; ++i) a.fref[i] = (float)((i == 0 ? P.phi1 : 0.0) + h->lc.F[i] * p0ref);
    a.walls = P.walls ? 1 : 0;
    a.visc_fixed = (P.visc_mode == DL_VISC_FIXED) ? 1 : 0;
    a.force = h->force32;
    const FastSpectral& fs = h->fsp;
    a.nm = fs.nm;
    a.modes = fs.d_modes;
    a.kx_off = fs.d_kxoff;
    a.twx = fs.d_tw[0];
    a.twy = fs.d_tw[1];
    a.twz = fs.d_tw[2];
    a.acc = fs.d_acc;
    a.fh = fs.d_fh[fs.par];
    a.fh_next = fs.d_fh[1 - fs.par];
    a.half_eps = 0.5 * P.eps;
    a.invN = 1.0 / ((double)h->nx * (double)h->ny * (double)h->nz);
}

static inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// band mode list (half spectrum kz >= 0, 1 <= |k|^2 < kc^2) sorted by kx, and
// e^{i 2 pi m / n} tables, for the in-kernel forcing
static int fast_spectral_alloc(dl_handle* h) {
    FastSpectral& fs = h->fsp;
    memset(&fs, 0, sizeof(fs));
    const int K = h->P.kc - 1;
    if (K < 1 || K > SK) return DL_OK;  // kc > 3: separate forcing launches
    if (2 * K + 1 > h->nx || 2 * K + 1 > h->ny || K + 1 > h->nz / 2) return DL_OK;  // band does not fit
    std::vector<int4> modes;
    std::vector<int> off(SNK + 1, 0);
    for (int kx = -SK; kx <= SK; ++kx) {
        off[kx + SK] = (int)modes.size();
        for (int kz = 0; kz <= K; ++kz)
            for (int ky = -K; ky <= K; ++ky) {
                const int kk = kx * kx + ky * ky + kz * kz;
                if (kk >= 1 && kk < h->P.kc * h->P.kc) modes.push_back(make_int4(kx, ky, kz, kz == 0 ? 1 : 2));
            }
    }
    off[SNK] = (int)modes.size();
    if ((int)modes.size() > SMAXM) return DL_OK;
    fs.nm = (int)modes.size();
    DL_CUDA(h, cudaMalloc(&fs.d_modes, sizeof(int4) * fs.nm));
    DL_CUDA(h, cudaMemcpy(fs.d_modes, modes.data(), sizeof(int4) * fs.nm, cudaMemcpyHostToDevice));
    DL_CUDA(h, cudaMalloc(&fs.d_kxoff, sizeof(int) * (SNK + 1)));
    DL_CUDA(h, cudaMemcpy(fs.d_kxoff, off.data(), sizeof(int) * (SNK + 1), cudaMemcpyHostToDevice));
    const int ns[3] = {h->nx, h->ny, h->nz};
    const double pi = acos(-1.0);
    for (int d = 0; d < 3; ++d) {
        std::vector<float2> t(ns[d]);
        for (int m = 0; m < ns[d]; ++m)
            t[m] = make_float2((float)cos(2.0 * pi * m / ns[d]), (float)sin(2.0 * pi * m / ns[d]));
        DL_CUDA(h, cudaMalloc(&fs.d_tw[d], sizeof(float2) * ns[d]));
        DL_CUDA(h, cudaMemcpy(fs.d_tw[d], t.data(), sizeof(float2) * ns[d], cudaMemcpyHostToDevice));
    }
    for (int k = 0; k < 2; ++k) {
        DL_CUDA(h, cudaMalloc(&fs.d_fh[k], sizeof(float2) * 3 * fs.nm));
        DL_CUDA(h, cudaMemset(fs.d_fh[k], 0, sizeof(float2) * 3 * fs.nm));
    }
    DL_CUDA(h, cudaMalloc(&fs.d_acc, sizeof(double) * 2 * 3 * fs.nm * SP_NREP));
    DL_CUDA(h, cudaMemset(fs.d_acc, 0, sizeof(double) * 2 * 3 * fs.nm * SP_NREP));
    fs.dirty = 1;
    return DL_OK;
}

static void fast_spectral_free(dl_handle* h) {
    FastSpectral& fs = h->fsp;
    cudaFree(fs.d_modes);
    cudaFree(fs.d_kxoff);
    for (int d = 0; d < 3; ++d) cudaFree(fs.d_tw[d]);
    for (int k = 0; k < 2; ++k) cudaFree(fs.d_fh[k]);
    cudaFree(fs.d_acc);
    memset(&fs, 0, sizeof(fs));
}

int fast_alloc(dl_handle* h) {
    const size_t N = h->N;
    const size_t es = (h->form == DL_FORM_FP16) ? sizeof(__half) : sizeof(float);
    for (int k = 0; k < 2; ++k) {
        if (!h->single) {  // the single-phase step has no f
            DL_CUDA(h, cudaMalloc(&h->fs[k], es * Q * N));
            DL_CUDA(h, cudaMemsetAsync(h->fs[k], 0, es * Q * N, h->stream));
        }
        DL_CUDA(h, cudaMalloc(&h->gs[k], es * Q * N));
        DL_CUDA(h, cudaMalloc(&h->mac32[k], sizeof(float) * 5 * N));
        DL_CUDA(h, cudaMemsetAsync(h->gs[k], 0, es * Q * N, h->stream));
        DL_CUDA(h, cudaMemsetAsync(h->mac32[k], 0, sizeof(float) * 5 * N, h->stream));
    }
    if (h->lz <= 0) h->lz = std::min(h->nz, DL_DEFAULT_LZ);
    return fast_spectral_alloc(h);
}

// the force arrays are only needed for a static force or kc > 3
static int ensure_force32(dl_handle* h) {
    if (h->force32) return DL_OK;
    DL_CUDA(h, cudaMalloc(&h->force32, sizeof(float) * 3 * h->N));
    DL_CUDA(h, cudaMemsetAsync(h->force32, 0, sizeof(float) * 3 * h->N, h->stream));
    return DL_OK;
}

int fast_prepare_force(dl_handle* h, int mode) {
    if (mode == DL_FORCE_STATIC || (mode == DL_FORCE_SPECTRAL && h->fsp.nm == 0)) return ensure_force32(h);
    if (mode == DL_FORCE_SPECTRAL) h->fsp.dirty = 1;
    return DL_OK;
}

void fast_free(dl_handle* h) {
    for (int k = 0; k < 2; ++k) {
        cudaFree(h->fs[k]);
        cudaFree(h->gs[k]);
        cudaFree(h->mac32[k]);
        h->fs[k] = h->gs[k] = nullptr;
        h->mac32[k] = nullptr;
    }
    h->push_tmap_ok = 0;  // the tensor maps name the freed buffers
    cudaFree(h->force32);
    h->force32 = nullptr;
    fast_spectral_free(h);
}

int fast_set_fields(dl_handle* h, const double* d_fields) {
    fields_to_fast<<<nblk(h->N, 256), 256, 0, h->stream>>>(d_fields, h->mac32[h->cur], (long long)h->N, h->P.phi1);
    DL_CUDA(h, cudaGetLastError());
    h->fsp.dirty = 1;
    return DL_OK;
}

int fast_get_fields(dl_handle* h, double* d_fields) {
    fast_to_fields<<<nblk(h->N, 256), 256, 0, h->stream>>>(h->mac32[h->cur], d_fields, (long long)h->N, h->P.phi1);
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int fast_init_equilibrium(dl_handle* h) {
    FastArgs a;
    fill_fast(h, a);
    a.mac = h->mac32[h->cur];
    a.fo = h->fs[h->cur];
    a.go = h->gs[h->cur];
    if (h->form == DL_FORM_FP16) DL_LAUNCH(h, false, (init_fast<__half, true><<<nblk(a.N, 256), 256, 0, h->stream>>>(a)));
    else DL_LAUNCH(h, false, (init_fast<float, false><<<nblk(a.N, 256), 256, 0, h->stream>>>(a)));
    DL_CUDA(h, cudaGetLastError());
    h->fsp.dirty = 1;
    return DL_OK;
}

int fast_get_populations(dl_handle* h, double* d_f, double* d_g) {
    FastArgs a;
    fill_fast(h, a);
    a.mac = h->mac32[h->cur];
    a.f = h->fs[h->cur];
    a.g = h->gs[h->cur];
    if (h->form == DL_FORM_FP16) pops_to_host<__half, true><<<nblk(a.N, 256), 256, 0, h->stream>>>(a, d_f, d_g);
    else pops_to_host<float, false><<<nblk(a.N, 256), 256, 0, h->stream>>>(a, d_f, d_g);
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int fast_set_populations(dl_handle* h, const double* d_f, const double* d_g) {
    FastArgs a;
    fill_fast(h, a);
    a.maco = h->mac32[h->cur];
    a.fo = h->fs[h->cur];
    a.go = h->gs[h->cur];
    if (h->form == DL_FORM_FP16) pops_from_host<__half, true><<<nblk(a.N, 256), 256, 0, h->stream>>>(a, d_f, d_g);
    else pops_from_host<float, false><<<nblk(a.N, 256), 256, 0, h->stream>>>(a, d_f, d_g);
    DL_CUDA(h, cudaGetLastError());
    h->fsp.dirty = 1;
    return DL_OK;
}

// band coefficients from the current u (first step after new fields)
static int fast_spectral_project(dl_handle* h) {
    const float* m = h->mac32[h->cur];
    int rc = spectral_project_f32(h, m + h->N, m + 2 * h->N, m + 3 * h->N);
    if (rc != DL_OK) return rc;
    FastSpectral& fs = h->fsp;
    DL_LAUNCH(h, false, (sp_fhat_from_uh<<<1, 256, 0, h->stream>>>(h->sp.d_uh, h->sp.K, fs.d_modes, fs.nm,
                                                                  0.5 * h->P.eps, fs.d_fh[fs.par], h->d_state)));
    DL_CUDA(h, cudaMemsetAsync(fs.d_acc, 0, sizeof(double) * 2 * 3 * fs.nm * SP_NREP, h->stream));
    DL_CUDA(h, cudaGetLastError());
    fs.dirty = 0;
    return DL_OK;
}

static const int PROJ_ROWS = 64;  // rows of the band projection per block (batched ensembles)

static int sm_count(dl_handle* h) {
    static int sms_of[64] = {0};
    int& sms = sms_of[h->device & 63];
    if (sms == 0 && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess) sms = 152;
    return sms;
}

// band projection launch: four blocks on every SM (the register limit), one
// wave; fewer blocks when there are fewer rows than warps
static int launch_projection(dl_handle* h, const FastArgs& a) {
    const long long rows = (long long)a.ny * a.nz;
    const int sms = sm_count(h);
    const long long need = (rows + PROJ_NT / 32 - 1) / (PROJ_NT / 32);
    const unsigned grid = (unsigned)std::min<long long>(4LL * sms, need);
    DL_LAUNCH(h, false, (sp_project_fast<<<grid, PROJ_NT, 0, h->stream>>>(a)));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

template <typename ST, bool RES, bool LES, int FMODE, bool SP = false>
static int launch_fused(dl_handle* h, const FastArgs& a) {
    static bool configured[64] = {false};
    static bool configured_pipe[64] = {false};
    const int dev = h->device & 63;
    const size_t sm = smem_bytes<RES, LES, FMODE, SP>();
    const bool pipe = SP && h->sp_pipeline;
    if (!(pipe ? configured_pipe[dev] : configured[dev])) {
        if constexpr (SP) {
            if (pipe)
                DL_CUDA(h, cudaFuncSetAttribute(step_fused_sp_pipe<ST, RES, FMODE>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            else
                DL_CUDA(h, cudaFuncSetAttribute(step_fused_sp<ST, RES, FMODE>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        } else {
            DL_CUDA(h, cudaFuncSetAttribute(step_fused<ST, RES, LES, FMODE>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        }
        (pipe ? configured_pipe[dev] : configured[dev]) = true;
    }
    dim3 grid((a.nx + TX - 1) / TX, (a.ny + TY - 1) / TY, (a.nz + a.lz - 1) / a.lz);
    if constexpr (SP) {
        if (pipe) DL_LAUNCH(h, true, (step_fused_sp_pipe<ST, RES, FMODE><<<grid, NT, sm, h->stream>>>(a)));
        else DL_LAUNCH(h, true, (step_fused_sp<ST, RES, FMODE><<<grid, NT, sm, h->stream>>>(a)));
    } else {
        DL_LAUNCH(h, true, (step_fused<ST, RES, LES, FMODE><<<grid, NT, sm, h->stream>>>(a)));
    }
    DL_CUDA(h, cudaGetLastError());
    if (FMODE == F_SPECTRAL && !a.proj_in_step) return launch_projection(h, a);
    return DL_OK;
}

template <typename ST, bool RES>
static int dispatch_single(dl_handle* h, const FastArgs& a, int fmode) {
    if (fmode == F_SPECTRAL) return launch_fused<ST, RES, false, F_SPECTRAL, true>(h, a);
    if (fmode == F_ARRAY) return launch_fused<ST, RES, false, F_ARRAY, true>(h, a);
    return launch_fused<ST, RES, false, F_NONE, true>(h, a);
}

template <typename ST, bool RES>
static int dispatch(dl_handle* h, const FastArgs& a, bool les, int fmode) {
    if (les) {
        if (fmode == F_SPECTRAL) return launch_fused<ST, RES, true, F_SPECTRAL>(h, a);
        if (fmode == F_ARRAY) return launch_fused<ST, RES, true, F_ARRAY>(h, a);
        return launch_fused<ST, RES, true, F_NONE>(h, a);
    }
    if (fmode == F_SPECTRAL) return launch_fused<ST, RES, false, F_SPECTRAL>(h, a);
    if (fmode == F_ARRAY) return launch_fused<ST, RES, false, F_ARRAY>(h, a);
    return launch_fused<ST, RES, false, F_NONE>(h, a);
}

// Step arguments of handle h for the state k steps ahead (k = 0 or 1):
// buffers, band coefficients and wall terms of that step.
int force_fmode(const dl_handle* h) {
    if (h->force_mode == DL_FORCE_STATIC) return F_ARRAY;
    if (h->force_mode == DL_FORCE_SPECTRAL) return h->fsp.nm > 0 ? F_SPECTRAL : F_ARRAY;
    return F_NONE;
}

// the moving-wall terms 6 E_j c_j . U_wall of bounce_back_LBM
// (prototype_program/two-phase/drop8_mpi.f90:651-671) for step `step`: the
// walls move from wall_start on
void wall_terms(const dl_handle* h, long long step, float* bot, float* top) {
    double U[3] = {0.0, 0.0, 0.0};
    if (step >= h->P.wall_start)
        for (int q = 0; q < 3; ++q) U[q] = h->P.wall_u[q];
    const int bot_src[5] = {6, 11, 12, 13, 10}, top_src[5] = {3, 14, 7, 8, 9};
    for (int q = 0; q < 5; ++q) {
        int j = bot_src[q];
        bot[q] = (float)(6.0 * h->lc.E[j] * ((-U[0]) * cx(j) + (-U[1]) * cy(j) + (-U[2]) * cz(j)));
        j = top_src[q];
        top[q] = (float)(6.0 * h->lc.E[j] * (U[0] * cx(j) + U[1] * cy(j) + U[2] * cz(j)));
    }
}

static void make_step_args(dl_handle* h, int k, FastArgs& a) {
    const int c = h->cur ^ k, n = 1 - c;
    const long long step = h->step + 1 + k;
    fill_fast(h, a);
    a.fh = h->fsp.d_fh[h->fsp.par ^ k];
    a.fh_next = h->fsp.d_fh[1 - (h->fsp.par ^ k)];
    a.mac = h->mac32[c];
    a.maco = h->mac32[n];
    a.f = h->fs[c];
    a.g = h->gs[c];
    a.fo = h->fs[n];
    a.go = h->gs[n];
    a.step = step;
    wall_terms(h, step, a.wall_bot, a.wall_top);
}

// work that must precede a fused step: band coefficients of new fields, or
// the force arrays of the separate-launch spectral path
static int pre_step(dl_handle* h) {
    if (h->force_mode != DL_FORCE_SPECTRAL) return DL_OK;
    if (h->fsp.nm > 0) return h->fsp.dirty ? fast_spectral_project(h) : DL_OK;
    const float* m = h->mac32[h->cur];
    return spectral_force_f32(h, m + h->N, m + 2 * h->N, m + 3 * h->N, h->force32, h->force32 + h->N,
                              h->force32 + 2 * h->N);
}

void advance(dl_handle* h, int n) {
    if (n & 1) {
        h->cur = 1 - h->cur;
        if (force_fmode(h) == F_SPECTRAL) h->fsp.par = 1 - h->fsp.par;
    }
    h->step += n;
}

int fast_step(dl_handle* h) {
    if (push_eligible(h)) return push_step(h);
    if (h->pushed) {
        const int src = fast_settle(h);
        if (src != DL_OK) return src;
    }
    int rc = pre_step(h);
    if (rc != DL_OK) return rc;
    FastArgs a;
    make_step_args(h, 0, a);
    const int fmode = force_fmode(h);
    const bool les = h->P.les != 0;
    if (h->single)
        rc = (h->form == DL_FORM_FP16) ? dispatch_single<__half, true>(h, a, fmode) : dispatch_single<float, false>(h, a, fmode);
    else
        rc = (h->form == DL_FORM_FP16) ? dispatch<__half, true>(h, a, les, fmode) : dispatch<float, false>(h, a, les, fmode);
    if (rc != DL_OK) return rc;
    advance(h, 1);
    return DL_OK;
}

// ---- batched ensembles ----------------------------------------------------------
// Two modes (batch option "persistent"). Default: every member takes its own
// one-launch steps on one of up to BATCH_WORKERS streams (batch_step_concurrent).
// Persistent: every member's tiles are work items of ONE persistent launch per
// step; each block copies its member's arguments into shared memory and runs
// the same fused body; each member keeps its own reduction state, so its last
// block finalises it. Optionally two steps are captured in a CUDA graph and
// replayed. (The persistent kernel is the slower of the two: its arguments in
// shared memory cost it registers, and its band projection is a launch of its
// own.)
template <typename ST, bool RES, bool LES, int FMODE>
__global__ void __launch_bounds__(NT, 2) step_batched(const FastArgs* __restrict__ table,
                                                      const int4* __restrict__ items, int nitems,
                                                      const unsigned* __restrict__ nblk_of) {
    extern __shared__ float smem[];
    __shared__ __align__(16) FastArgs s_a;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        __syncthreads();
        const int4 it = items[w];
        const int* src = (const int*)(table + it.x);
        int* dst = (int*)&s_a;
        for (int t = threadIdx.x; t < (int)(sizeof(FastArgs) / sizeof(int)); t += blockDim.x) dst[t] = src[t];
        __syncthreads();
        float bmin = INFINITY, bmax = -INFINITY;
        bool bad = false;
        const int z0 = it.w * s_a.lz;
        fused_body<ST, RES, LES, FMODE, false>(s_a, smem, it.y, it.z, z0, min(z0 + s_a.lz, s_a.nz), bmin, bmax, bad);
        minmax_block_and_finalize<float>(s_a.st, (double)bmin, (double)bmax, s_a.maco, s_a.phi1, s_a.N,
                                         (double)s_a.phi1, (double)s_a.phi2, bad, s_a.step, nblk_of[it.x]);
    }
}

// band projection of every member's new u: work items (member, first row)
__global__ void __launch_bounds__(PROJ_NT) sp_project_batched(const FastArgs* __restrict__ table,
                                                              const int2* __restrict__ items, int nitems,
                                                              const unsigned* __restrict__ nblk_of, int rows_per_item) {
    __shared__ __align__(16) FastArgs s_a;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        __syncthreads();
        const int2 it = items[w];
        const int* src = (const int*)(table + it.x);
        int* dst = (int*)&s_a;
        for (int t = threadIdx.x; t < (int)(sizeof(FastArgs) / sizeof(int)); t += blockDim.x) dst[t] = src[t];
        __syncthreads();
        const int rows = s_a.ny * s_a.nz;
        const int r0 = it.y * rows_per_item;
        project_rows(s_a, r0 + (threadIdx.x >> 5), PROJ_NT / 32, min(r0 + rows_per_item, rows), nblk_of[it.x]);
    }
}

constexpr int BATCH_WORKERS = 16;  // concurrent mode: streams the members' steps are spread over

struct BatchImpl {
    int nm;
    int form;
    dl_handle** mem;
    FastArgs* h_table;      // [2][nm] host copy
    FastArgs* d_table;      // [2][nm]
    int4* d_items;
    unsigned* d_nblk;
    int nitems;
    int2* d_pitems;         // projection work items (member, row block)
    unsigned* d_pnblk;      // projection blocks per member
    int npitems;
    int lz, bps, use_graph;
    int persistent;         // 1: one persistent launch per step over all members; 0: the members' own steps, concurrent
    int nworkers;           // concurrent mode: worker streams (created on first use)
    cudaStream_t workers[BATCH_WORKERS];
    cudaEvent_t fork, join[BATCH_WORKERS];
    int sms;
    cudaStream_t stream;
    cudaStream_t cap_stream;  // owned stream the graph is captured on (the legacy default stream cannot capture)
    cudaGraphExec_t gexec;
    int graph_ok;
    int built_parity;       // member parity the tables were built at (-1: rebuild)
    int fmode, les;
    int push;               // persistent mode in the push form (every member push-eligible)
    int built_push;         // the form the tables were built for
    unsigned char* h_ptable;  // push form: [2][nm] step arguments (host copy)
    void* d_ptable;
    unsigned* d_counter;    // push form: the launch's next work item
};

template <typename ST, bool RES, bool LES, int FMODE>
static int launch_batched_t(dl_handle* h0, BatchImpl* b, int k) {
    static bool configured[64] = {false};
    const int dev = h0->device & 63;
    const size_t sm = smem_bytes<RES, LES, FMODE>();
    if (!configured[dev]) {
        DL_CUDA(h0, cudaFuncSetAttribute(step_batched<ST, RES, LES, FMODE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        configured[dev] = true;
    }
    const int grid = min(b->nitems, b->bps * b->sms);
    step_batched<ST, RES, LES, FMODE><<<grid, NT, sm, b->stream>>>(b->d_table + (size_t)k * b->nm, b->d_items,
                                                                  b->nitems, b->d_nblk);
    DL_CUDA(h0, cudaGetLastError());
    if (FMODE == F_SPECTRAL) {
        const int pg = min(b->npitems, 4 * b->sms);
        sp_project_batched<<<pg, PROJ_NT, 0, b->stream>>>(b->d_table + (size_t)k * b->nm, b->d_pitems, b->npitems,
                                                          b->d_pnblk, PROJ_ROWS);
        DL_CUDA(h0, cudaGetLastError());
    }
    return DL_OK;
}

template <typename ST, bool RES>
static int launch_batched_st(dl_handle* h0, BatchImpl* b, int k) {
    if (b->les) {
        if (b->fmode == F_SPECTRAL) return launch_batched_t<ST, RES, true, F_SPECTRAL>(h0, b, k);
        if (b->fmode == F_ARRAY) return launch_batched_t<ST, RES, true, F_ARRAY>(h0, b, k);
        return launch_batched_t<ST, RES, true, F_NONE>(h0, b, k);
    }
    if (b->fmode == F_SPECTRAL) return launch_batched_t<ST, RES, false, F_SPECTRAL>(h0, b, k);
    if (b->fmode == F_ARRAY) return launch_batched_t<ST, RES, false, F_ARRAY>(h0, b, k);
    return launch_batched_t<ST, RES, false, F_NONE>(h0, b, k);
}

static int launch_batched(BatchImpl* b, int k) {
    dl_handle* h0 = b->mem[0];
    if (b->push) {
        const int grid = min(b->nitems, b->bps * b->sms);
        return launch_push_batched(h0, (const unsigned char*)b->d_ptable + (size_t)k * b->nm * push_args_bytes(),
                                   b->nm, b->d_items, b->nitems, b->d_nblk, b->d_counter, grid, b->stream);
    }
    return b->form == DL_FORM_FP16 ? launch_batched_st<__half, true>(h0, b, k) : launch_batched_st<float, false>(h0, b, k);
}

int batch_create(dl_handle** members, int nm, void** out) {
    dl_handle* h0 = members[0];
    BatchImpl* b = (BatchImpl*)calloc(1, sizeof(BatchImpl));
    if (!b) return DL_ERR_ALLOC;
    b->nm = nm;
    b->form = h0->form;
    b->mem = members;
    b->lz = DL_DEFAULT_LZ;
    b->bps = 2;
    b->use_graph = 1;
    b->persistent = 0;
    b->stream = h0->stream;
    b->built_parity = -1;
    b->les = h0->P.les != 0;
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, h0->device);
    b->h_table = (FastArgs*)calloc(2 * (size_t)nm, sizeof(FastArgs));
    if (!b->h_table) {
        free(b);
        return DL_ERR_ALLOC;
    }
    if (cudaMalloc(&b->d_table, 2 * (size_t)nm * sizeof(FastArgs)) != cudaSuccess ||
        cudaMalloc(&b->d_nblk, (size_t)nm * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&b->d_pnblk, (size_t)nm * sizeof(unsigned)) != cudaSuccess) {
        batch_destroy(b);
        return DL_ERR_ALLOC;
    }
    *out = b;
    return DL_OK;
}

void batch_destroy(void* p) {
    BatchImpl* b = (BatchImpl*)p;
    if (!b) return;
    if (b->graph_ok) cudaGraphExecDestroy(b->gexec);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    for (int w = 0; w < b->nworkers; ++w) {
        cudaStreamDestroy(b->workers[w]);
        cudaEventDestroy(b->join[w]);
    }
    if (b->nworkers) cudaEventDestroy(b->fork);
    cudaFree(b->d_table);
    cudaFree(b->d_items);
    cudaFree(b->d_nblk);
    cudaFree(b->d_pitems);
    cudaFree(b->d_pnblk);
    cudaFree(b->d_ptable);
    cudaFree(b->d_counter);
    free(b->h_table);
    free(b->h_ptable);
    free(b);
}

int batch_set_option(void* p, const char* key, long long v) {
    BatchImpl* b = (BatchImpl*)p;
    if (strcmp(key, "lz") == 0) {
        if (v < 1 || v > 4096) return DL_ERR_ARG;
        b->lz = (int)v;
    } else if (strcmp(key, "blocks_per_sm") == 0) {
        if (v < 1 || v > 2) return DL_ERR_ARG;
        b->bps = (int)v;
    } else if (strcmp(key, "graph") == 0) {
        b->use_graph = v ? 1 : 0;
    } else if (strcmp(key, "persistent") == 0) {
        if (v < 0 || v > 1) return DL_ERR_ARG;
        b->persistent = (int)v;
    } else {
        return DL_ERR_ARG;
    }
    b->built_parity = -1;  // rebuild tables, items and graph
    return DL_OK;
}

int batch_get_option(void* p, const char* key, long long* v) {
    BatchImpl* b = (BatchImpl*)p;
    if (strcmp(key, "lz") == 0) *v = b->lz;
    else if (strcmp(key, "blocks_per_sm") == 0) *v = b->bps;
    else if (strcmp(key, "graph") == 0) *v = b->use_graph;
    else if (strcmp(key, "persistent") == 0) *v = b->persistent;
    else return DL_ERR_ARG;
    return DL_OK;
}

// (re)build the two argument tables (this step and the next), the work items
// and the graph for the members' current state
static int batch_build(BatchImpl* b) {
    dl_handle* h0 = b->mem[0];
    const int nm = b->nm;
    b->fmode = force_fmode(h0);
    std::vector<int4> items;
    std::vector<unsigned> nblk(nm);
    // largest members first: their items are the longest
    std::vector<int> order(nm);
    for (int m = 0; m < nm; ++m) order[m] = m;
    for (int i = 1; i < nm; ++i)
        for (int j = i; j > 0 && b->mem[order[j]]->N > b->mem[order[j - 1]]->N; --j) std::swap(order[j], order[j - 1]);
    const size_t psz = push_args_bytes();
    if (b->push && !b->h_ptable) {
        b->h_ptable = (unsigned char*)calloc(2 * (size_t)nm, psz);
        if (!b->h_ptable) return set_error(h0, DL_ERR_ALLOC, "batch argument table");
        DL_CUDA(h0, cudaMalloc(&b->d_ptable, 2 * (size_t)nm * psz));
        DL_CUDA(h0, cudaMalloc(&b->d_counter, sizeof(unsigned)));
    }
    for (int m = 0; m < nm; ++m) {
        dl_handle* h = b->mem[m];
        h->lz = min(b->lz, h->nz);
        for (int k = 0; k < 2; ++k) {
            if (b->push) {
                push_args_at(h, k, b->h_ptable + ((size_t)k * nm + m) * psz);  // the projection is in the push body
            } else {
                make_step_args(h, k, b->h_table[(size_t)k * nm + m]);
                b->h_table[(size_t)k * nm + m].proj_in_step = 0;  // the batch projects in its own launch
            }
        }
        const int gx = (h->nx + TX - 1) / TX, gy = (h->ny + TY - 1) / TY, gz = (h->nz + h->lz - 1) / h->lz;
        nblk[m] = (unsigned)(gx * gy * gz);
    }
    for (int oi = 0; oi < nm; ++oi) {
        const int m = order[oi];
        dl_handle* h = b->mem[m];
        const int gx = (h->nx + TX - 1) / TX, gy = (h->ny + TY - 1) / TY, gz = (h->nz + h->lz - 1) / h->lz;
        for (int bz = 0; bz < gz; ++bz)
            for (int by = 0; by < gy; ++by)
                for (int bx = 0; bx < gx; ++bx) items.push_back(make_int4(m, bx, by, bz));
    }
    if ((int)items.size() != b->nitems || !b->d_items) {
        cudaFree(b->d_items);
        b->d_items = nullptr;
        DL_CUDA(h0, cudaMalloc(&b->d_items, items.size() * sizeof(int4)));
    }
    b->nitems = (int)items.size();
    DL_CUDA(h0, cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
    // projection items: every member's rows in blocks of PROJ_ROWS
    std::vector<int2> pitems;
    std::vector<unsigned> pnblk(nm);
    for (int m = 0; m < nm; ++m) {
        const long long rows = (long long)b->mem[m]->ny * b->mem[m]->nz;
        const int nb = (int)((rows + PROJ_ROWS - 1) / PROJ_ROWS);
        pnblk[m] = (unsigned)nb;
        for (int r = 0; r < nb; ++r) pitems.push_back(make_int2(m, r));
    }
    if ((int)pitems.size() != b->npitems || !b->d_pitems) {
        cudaFree(b->d_pitems);
        b->d_pitems = nullptr;
        DL_CUDA(h0, cudaMalloc(&b->d_pitems, pitems.size() * sizeof(int2)));
    }
    b->npitems = (int)pitems.size();
    DL_CUDA(h0, cudaMemcpyAsync(b->d_pitems, pitems.data(), pitems.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                b->stream));
    DL_CUDA(h0, cudaMemcpyAsync(b->d_pnblk, pnblk.data(), nm * sizeof(unsigned), cudaMemcpyHostToDevice, b->stream));
    DL_CUDA(h0, cudaMemcpyAsync(b->d_nblk, nblk.data(), nm * sizeof(unsigned), cudaMemcpyHostToDevice, b->stream));
    DL_CUDA(h0, cudaMemcpyAsync(b->d_table, b->h_table, 2 * (size_t)nm * sizeof(FastArgs), cudaMemcpyHostToDevice,
                                b->stream));
    if (b->push)
        DL_CUDA(h0, cudaMemcpyAsync(b->d_ptable, b->h_ptable, 2 * (size_t)nm * psz, cudaMemcpyHostToDevice, b->stream));
    DL_CUDA(h0, cudaStreamSynchronize(b->stream));
    if (b->graph_ok) {
        cudaGraphExecDestroy(b->gexec);
        b->graph_ok = 0;
    }
    if (b->use_graph) {
        // capture on the batch's own stream, replay on the caller's stream
        if (!b->cap_stream) DL_CUDA(h0, cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
        cudaGraph_t g;
        const cudaStream_t user = b->stream;
        b->stream = b->cap_stream;
        cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) {
            b->stream = user;
            return check_cuda(h0, e, "cudaStreamBeginCapture");
        }
        int rc = launch_batched(b, 0);
        if (rc == DL_OK) rc = launch_batched(b, 1);
        e = cudaStreamEndCapture(b->stream, &g);
        b->stream = user;
        if (rc != DL_OK) return rc;
        DL_CUDA(h0, e);
        e = cudaGraphInstantiate(&b->gexec, g, 0);
        cudaGraphDestroy(g);
        DL_CUDA(h0, e);
        b->graph_ok = 1;
    }
    b->built_parity = h0->cur;
    b->built_push = b->push;
    return DL_OK;
}

// concurrent mode: every member takes its own one-launch steps (the single-
// handle path, kernel arguments in constant memory, band projection in the
// step) on one of up to BATCH_WORKERS streams forked from member 0's stream
// and joined back to it at the end; members of any size, parity and force mode
static int batch_step_concurrent(BatchImpl* b, int nsteps) {
    dl_handle* h0 = b->mem[0];
    const int nm = b->nm;
    for (int m = 0; m < nm; ++m)
        if (!b->mem[m]->eq_init) return set_error(h0, DL_ERR_STATE, "member %d not initialised", m);
    if (!b->nworkers) {
        const int nw = std::min(nm, BATCH_WORKERS);
        DL_CUDA(h0, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
        for (int w = 0; w < nw; ++w) {
            DL_CUDA(h0, cudaStreamCreateWithFlags(&b->workers[w], cudaStreamNonBlocking));
            DL_CUDA(h0, cudaEventCreateWithFlags(&b->join[w], cudaEventDisableTiming));
            b->nworkers = w + 1;
        }
    }
    const int nw = b->nworkers;
    cudaStream_t home = h0->stream;
    DL_CUDA(h0, cudaEventRecord(b->fork, home));
    for (int w = 0; w < nw; ++w) DL_CUDA(h0, cudaStreamWaitEvent(b->workers[w], b->fork, 0));
    // a member with a stream of its own: its worker also waits for that stream
    // (work the caller enqueued there, e.g. set-up copies)
    for (int m = 0; m < nm; ++m)
        if (b->mem[m]->stream != home) {
            DL_CUDA(h0, cudaEventRecord(b->fork, b->mem[m]->stream));
            DL_CUDA(h0, cudaStreamWaitEvent(b->workers[m % nw], b->fork, 0));
        }
    int rc = DL_OK;
    for (int s = 0; s < nsteps && rc == DL_OK; ++s)
        for (int m = 0; m < nm && rc == DL_OK; ++m) {
            dl_handle* h = b->mem[m];
            h->lz = std::min(b->lz, h->nz);
            cudaStream_t own = h->stream;
            h->stream = b->workers[m % nw];
            rc = fast_step(h);
            h->stream = own;
        }
    // join even after an error, so that the home stream (and a member's own stream)
    // never runs ahead of the workers
    for (int w = 0; w < nw; ++w) {
        DL_CUDA(h0, cudaEventRecord(b->join[w], b->workers[w]));
        DL_CUDA(h0, cudaStreamWaitEvent(home, b->join[w], 0));
    }
    for (int m = 0; m < nm; ++m)
        if (b->mem[m]->stream != home) DL_CUDA(h0, cudaStreamWaitEvent(b->mem[m]->stream, b->join[m % nw], 0));
    return rc;
}

int batch_step(void* p, int nsteps) {
    BatchImpl* b = (BatchImpl*)p;
    if (!b->persistent) return batch_step_concurrent(b, nsteps);
    dl_handle* h0 = b->mem[0];
    const int nm = b->nm;
    // members step together: same parity and step count, same kernel variant
    for (int m = 0; m < nm; ++m) {
        dl_handle* h = b->mem[m];
        if (!h->eq_init) return set_error(h0, DL_ERR_STATE, "member %d not initialised", m);
        if (h->cur != h0->cur || h->step != h0->step || force_fmode(h) != force_fmode(h0) ||
            (h->fsp.par != h0->fsp.par && force_fmode(h) == F_SPECTRAL) || (h->P.les != 0) != (b->les != 0))
            return set_error(h0, DL_ERR_STATE, "member %d is not in step with member 0", m);
        if (h->P.walls && h->P.wall_start > h->step + 1 && h->P.wall_start <= h->step + nsteps)
            return set_error(h0, DL_ERR_UNSUPPORTED, "wall start inside a batched call; split the call");
    }
    // the push form when every member takes it (FP32 members); else the pull form
    bool push = true;
    for (int m = 0; m < nm; ++m) push = push && push_eligible(b->mem[m]);
    b->push = push ? 1 : 0;
    int left = nsteps;
    if (push) {
        // the captured steps load a push step's (pending) state: members that
        // are settled take one step of their own first, all of them, to stay in step
        bool settled_any = false;
        for (int m = 0; m < nm; ++m) settled_any = settled_any || !b->mem[m]->pushed;
        if (settled_any && left > 0) {
            for (int m = 0; m < nm; ++m) {
                dl_handle* h = b->mem[m];
                const cudaStream_t own = h->stream;
                h->stream = h0->stream;  // ordered before the persistent launches
                int rc = push_step(h);
                h->stream = own;
                if (rc != DL_OK) return rc;
            }
            left -= 1;
        }
    } else {
        for (int m = 0; m < nm; ++m) {
            int rc = fast_settle(b->mem[m]);  // the persistent launch steps the pull form
            if (rc != DL_OK) return rc;
        }
        for (int m = 0; m < nm; ++m) {
            const int dirty = b->mem[m]->fsp.dirty;
            int rc = pre_step(b->mem[m]);
            if (rc != DL_OK) return rc;
            if (dirty) b->built_parity = -1;
        }
    }
    if (b->built_parity < 0 || b->fmode != force_fmode(h0) || b->stream != h0->stream || b->built_push != b->push) {
        b->stream = h0->stream;
        int rc = batch_build(b);
        if (rc != DL_OK) return rc;
    }
    // table 0 is the step from the parity the tables were built at, table 1
    // the step after it; the graph runs table 0 then table 1. (The tables'
    // absolute step numbers only feed the NaN report and the wall terms,
    // which are constant inside one call.)
    auto stepped = [&](int n) {
        for (int m = 0; m < nm; ++m) {
            advance(b->mem[m], n);
            if (push) {
                b->mem[m]->pushed = 1;
                b->mem[m]->fsp.dirty = 0;
            }
        }
    };
    while (left > 0) {
        const int k = (h0->cur == b->built_parity) ? 0 : 1;
        if (b->graph_ok && k == 0 && left >= 2) {
            launch_begin(h0);
            DL_CUDA(h0, cudaGraphLaunch(b->gexec, b->stream));
            launch_end(h0, true);
            h0->launches += 1;  // the graph holds two step launches
            stepped(2);
            left -= 2;
        } else {
            launch_begin(h0);
            int rc = launch_batched(b, k);
            launch_end(h0, true);
            if (rc != DL_OK) return rc;
            stepped(1);
            left -= 1;
        }
    }
    return DL_OK;
}

}  // namespace dl
