// adjoint.cu -- hand-written adjoint (reverse mode) of the FP32 droplet step,
// for gradients of a loss on the final phi with respect to kappaf, kappag,
// tau_f (the mobility (tau_f - 1/2) ds), the wall velocity and the initial phi.
//
// Forward step being differentiated (program/lbm_drop_xy.f90:421-588 with the
// walls of prototype_program/two-phase/drop8_mpi.f90:642-674), at constant
// tau_g (viscosity ratio 1; see below for the per-site tau_g):
//   f'_i(x) = (1 - wf) f_i(x - c_i) + wf feq_i(x - c_i)
//   g'_i(x) = (1 - wg) g_i(x - c_i) + wg geq_i(x - c_i)   (+ a constant force)
//   wall nodes: g'_i = g'_j - 6 E_j (U_wall . c_j) for the reflected pairs
//   feq_i = H_i phi + F_i A + 3 E_i phi c_i.u + E_i kf cGc_i
//   geq_i = E_i (3p + 3 c_i.u + 4.5 (c_i.u)^2 - 1.5 u^2) + E_i kg cGc_i
//   A = p0(phi) - kf phi lap(phi) - kf/6 |grad phi|^2,
//   cGc_i = 4.5 (c_i.grad phi)^2 - 1.5 |c_i|^2 |grad phi|^2,
//   phi = sum f, p = sum g / 3, u = sum c g.
// With the Smagorinsky term (program/LES_drop_xy.f90:481-502, 663-690) wg is
// per site: tau_g = 1/2 + 3 (nu + nu_t)/ds, nu_t = csd sqrt(2 S:S), S the
// symmetric part of G_ab = d u_a / d x_b from the 14-neighbour stencil of u;
// its adjoint needs the pre-step g (the adjoint state then carries it) and
// sends dL/dG back to u through the transposed stencil. With a viscosity ratio
// other than 1 in the fixed-range mode (program/lbm_drop_xy.f90:254-285),
// nu = nu1 + (phi - phi1) (nu2 - nu1) / (phi2 - phi1) makes wg a function of
// the site's phi as well; dL/dwg then also reaches phi. With the band force
// (program/lbm_drop_iht_xy.f90:722-842), g'_i(x) gains 3 E_i c_i . F(x - c_i),
// F = (0.5 eps / E(u)) P u from the band projection P of the pre-step u:
// adj_local forms dL/dF(y) = sum_i 3 E_i c_i b_i(y) and spectral_adjoint_f32
// adds its pull-back onto u (through P and through E) to lu.
// Reverse of one step = three launches:
//   adj_walls   reflected adjoints at the wall planes, d/dU;
//   adj_local   per source site y: gather a_i = lf'_i(y + c_i), b_i = lg'_i(y + c_i)
//               and form the local adjoints of phi, A (-> lap, |grad|^2), grad phi,
//               u, p; d/dkf, d/dkg, d/dwf;
//   adj_stencil per site x: transpose of the lap/grad stencils (and, LES, of
//               the u stencil), then
//               lf_i = (1-wf) a_i + lphi, lg_i = (1-wg(x)) b_i + lp/3 + c_i.lu.
// States are in the FP32 form's layout: df[15][N] (deviations from the bulk
// equilibrium) followed by dphi, u1, u2, u3, dp [5][N] and, with LES, dg[15][N]
// (the adjoint state), or df, dg[15][N], fields (the full state of the initial
// step).
#include "dl_internal.cuh"
#include "dl_device.cuh"

#include <math.h>
#include <string.h>

namespace dl {

struct AdjArgs {
    int nx, ny, nz;
    unsigned N;
    const float* st;      // forward f before the step: df[15N]
    const float* mac;     // forward fields before the step: [5][N]
    const float* gst;     // LES: forward g before the step: dg[15N]
    const float* lin;     // adjoint of the post-step populations, [30][N] (f then g)
    float* lout;          // adjoint of the pre-step populations, [30][N]
    float* aux;           // [9][N]: lphi_loc, llap, lgrad x y z, lp, lu x y z; LES: + [9][N] dL/dG_ab
                          // (a + 3 b) and [1][N] wg
    double* grads;        // [ADJ_NREP][4]: d/dkf, d/dkg, d/dwf, d/dU (block b adds to copy b % ADJ_NREP)
    float phi1, omf, omg, kf, kf6, kg, T, a, b, inv_lap, inv_grad;
    float fref[Q];
    float wbot[5], wtop[5];   // d g'_i / dU at the bottom / top wall, per reflected pair
    int walls_on;             // the walls moved in this step
    int stream;               // 1: a time step; 0: the initial f = feq, g = geq
    int les;                  // Smagorinsky eddy viscosity in tau_g (time steps)
    float kvis;               // d nu / d phi: (nu2 - nu1) / (phi2 - phi1) (fixed range), 0 at ratio 1
    int spec;                 // band force (time steps): aux rows 19..21 receive dL/dF
    float csd, nu1, inv_ds;   // LES: (Cs delta)^2, nu, 1/ds
};
constexpr int ADJ_AUX = 22;  // aux rows: 9, LES dL/dG (9 .. 17), per-site wg (18), band force dL/dF (19 .. 21)

constexpr int ADJ_NREP = 64;  // copies of the gradient accumulators (spreads the atomics)

__device__ __forceinline__ int pmodi(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}
__device__ __forceinline__ constexpr float EW(int i) { return i == 0 ? 2.0f / 9.0f : (i <= 6 ? 1.0f / 9.0f : 1.0f / 72.0f); }
__device__ __forceinline__ constexpr float FW(int i) { return i == 0 ? -7.0f / 3.0f : (i <= 6 ? 1.0f / 3.0f : 1.0f / 24.0f); }
__device__ __forceinline__ constexpr float HW(int i) { return i == 0 ? 1.f : 0.f; }
__device__ __forceinline__ constexpr float C2(int i) { return i == 0 ? 0.f : (i <= 6 ? 1.f : 3.f); }

__device__ __forceinline__ unsigned nbr(const AdjArgs& a, int x, int y, int z, int dx, int dy, int dz) {
    return (unsigned)pmodi(x + dx, a.nx) + (unsigned)a.nx * ((unsigned)pmodi(y + dy, a.ny) + (unsigned)a.ny * (unsigned)pmodi(z + dz, a.nz));
}

template <int NV>
__device__ __forceinline__ void block_add(double (&v)[NV], double* out) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) sh[k][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[threadIdx.x][w];
        atomicAdd(out + threadIdx.x, s);
    }
}

// reflected pairs at the walls (reference i = 4,8,9,10,15 <- 7,12,13,14,11 at
// the bottom; 7,11,12,13,14 <- 4,15,8,9,10 at the top)
__global__ void adj_walls(AdjArgs a) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long plane = (long long)a.nx * a.ny;
    double dU = 0.0;
    if (t < 2 * plane && a.walls_on) {
        const bool top = t >= plane;
        const unsigned s = (unsigned)(t - (top ? plane : 0)) + (top ? (unsigned)(a.nz - 1) * (unsigned)plane : 0u);
        const int bi[5] = {3, 7, 8, 9, 14}, bj[5] = {6, 11, 12, 13, 10};
        const int ti[5] = {6, 10, 11, 12, 13}, tj[5] = {3, 14, 7, 8, 9};
        float* lg = a.lout + (size_t)Q * a.N;  // adjoints of g' (in place)
        for (int k = 0; k < 5; ++k) {
            const int i = top ? ti[k] : bi[k], j = top ? tj[k] : bj[k];
            const float li = lg[(size_t)i * a.N + s];
            lg[(size_t)j * a.N + s] += li;
            lg[(size_t)i * a.N + s] = 0.f;
            dU += (double)li * (double)(top ? a.wtop[k] : a.wbot[k]);
        }
    }
    double v[1] = {dU};
    block_add<1>(v, a.grads + 4 * (blockIdx.x % ADJ_NREP) + 3);
}

// PW: tau_g per site (LES and / or a viscosity ratio); LES: the Smagorinsky
// term; SPEC: the band force. The plain step takes <false, false, false>, the
// reverse of the initial equilibrium (no collision) too.
template <bool PW, bool LES, bool SPEC>
__global__ void __launch_bounds__(256) adj_local(AdjArgs a) {
    const long long s0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool active = s0 < (long long)a.N;
    const unsigned s = active ? (unsigned)s0 : 0u;
    const unsigned N = a.N;
    const int x = (int)(s % a.nx), y = (int)((s / a.nx) % a.ny), z = (int)(s / ((unsigned)a.nx * a.ny));
    const float* mac = a.mac;
    const float dphi = mac[s], u1 = mac[N + s], u2 = mac[2 * N + s], u3 = mac[3 * N + s];
    const float phi = a.phi1 + dphi;
    float v[Q];
#pragma unroll
    for (int i = 1; i < Q; ++i) v[i] = mac[nbr(a, x, y, z, cx(i), cy(i), cz(i))];
    float lap = -14.f * dphi;
#pragma unroll
    for (int i = 1; i < Q; ++i) lap += v[i];
    lap *= a.inv_lap;
    float gr[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        gr[0] += cx(i) * v[i];
        gr[1] += cy(i) * v[i];
        gr[2] += cz(i) * v[i];
    }
    gr[0] *= a.inv_grad;
    gr[1] *= a.inv_grad;
    gr[2] *= a.inv_grad;
    const float gsq = gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2];
    // p0(phi) - p0(phi1) and p0'(phi)
    const float omb = 1.f - a.b * phi;
    const float p0 = phi * a.T / omb - a.a * phi * phi;
    const float p0ref = a.phi1 * a.T / (1.f - a.b * a.phi1) - a.a * a.phi1 * a.phi1;
    const float dp0 = a.T / (omb * omb) - 2.f * a.a * phi;
    const float dA = (p0 - p0ref) - a.kf * phi * lap - a.kf6 * gsq;
    // per-site wg (LES and / or a viscosity ratio): G_ab = d u_a / d x_b, S, nu_t, nu(phi)
    const bool les = LES && a.stream;
    const bool pw = PW && a.stream;
    float G[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float tt = 0.f, wgs = a.omg, nut = 0.f;
    if (les) {
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const unsigned m = nbr(a, x, y, z, cx(k), cy(k), cz(k));
            const float uk[3] = {mac[N + m], mac[2 * N + m], mac[3 * N + m]};
#pragma unroll
            for (int al = 0; al < 3; ++al) {
                if (cx(k)) G[al][0] += cx(k) * uk[al];
                if (cy(k)) G[al][1] += cy(k) * uk[al];
                if (cz(k)) G[al][2] += cz(k) * uk[al];
            }
        }
        float acc = 0.f;
#pragma unroll
        for (int al = 0; al < 3; ++al)
#pragma unroll
            for (int be = 0; be < 3; ++be) {
                G[al][be] *= a.inv_grad;
            }
#pragma unroll
        for (int al = 0; al < 3; ++al)
#pragma unroll
            for (int be = 0; be < 3; ++be) {
                const float sab = 0.5f * (G[al][be] + G[be][al]);
                acc += sab * sab;
            }
        tt = 2.f * acc;
        nut = tt > 0.f ? a.csd * sqrtf(tt) : 0.f;
    }
    if (pw) wgs = 1.f / (0.5f + 3.f * (a.nu1 + dphi * a.kvis + nut) * a.inv_ds);
    float lw = 0.f;  // per-site wg: dL/dwg of this site
    float lF[3] = {0.f, 0.f, 0.f};  // band force: dL/dF of this site
    float lphi = 0.f, lA = 0.f, lp = 0.f, lusq = 0.f, lgsq = 0.f;
    float lu[3] = {0.f, 0.f, 0.f}, lgr[3] = {0.f, 0.f, 0.f};
    // per-site sums in FP32 (15 terms); FP64 from the block sums on (GB300's FP64 rate is low)
    float dkf = 0.f, dkg = 0.f, domf = 0.f;
    const float wf = a.stream ? a.omf : 1.f, wg = a.stream ? wgs : 1.f;
    const float dp = mac[4 * N + s];
    const float usq = u1 * u1 + u2 * u2 + u3 * u3;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const unsigned src = a.stream ? nbr(a, x, y, z, cx(i), cy(i), cz(i)) : s;
        const float ai = a.lin[(size_t)i * N + src];
        const float bi = a.lin[(size_t)(Q + i) * N + src];
        const float Lf = wf * ai, Lg = wg * bi;
        const float cu = cx(i) * u1 + cy(i) * u2 + cz(i) * u3;
        const float cg = cx(i) * gr[0] + cy(i) * gr[1] + cz(i) * gr[2];
        const float cGc = 4.5f * cg * cg - 1.5f * C2(i) * gsq;
        const float E = EW(i);
        if (a.stream) {
            const float dfeq = HW(i) * dphi + FW(i) * dA + E * (3.f * phi * cu + a.kf * cGc);
            domf += ai * (dfeq - a.st[(size_t)i * N + s]);
        }
        if (SPEC && a.stream) {
            lF[0] += 3.f * E * cx(i) * bi;
            lF[1] += 3.f * E * cy(i) * bi;
            lF[2] += 3.f * E * cz(i) * bi;
        }
        if (pw) {  // geq_i - g_i in deviations (the bulk E_i cancels)
            const float dgeq = E * (3.f * dp + 3.f * cu + 4.5f * cu * cu - 1.5f * usq + a.kg * cGc);
            lw += bi * (dgeq - a.gst[(size_t)i * N + s]);
        }
        lphi += Lf * (HW(i) + 3.f * E * cu);
        lA += Lf * FW(i);
        const float lcu = Lf * 3.f * E * phi + Lg * E * (3.f + 9.f * cu);
        const float lcGc = Lf * E * a.kf + Lg * E * a.kg;
        lp += Lg * 3.f * E;
        lusq -= 1.5f * Lg * E;
        dkf += Lf * E * cGc;
        dkg += Lg * E * cGc;
        lu[0] += lcu * cx(i);
        lu[1] += lcu * cy(i);
        lu[2] += lcu * cz(i);
        const float lcg = 9.f * cg * lcGc;
        lgsq -= 1.5f * C2(i) * lcGc;
        lgr[0] += lcg * cx(i);
        lgr[1] += lcg * cy(i);
        lgr[2] += lcg * cz(i);
    }
    lu[0] += 2.f * u1 * lusq;
    lu[1] += 2.f * u2 * lusq;
    lu[2] += 2.f * u3 * lusq;
    dkf += lA * (-phi * lap - gsq / 6.f);
    lphi += lA * (dp0 - a.kf * lap);
    const float lnu = pw ? lw * (-3.f * wgs * wgs * a.inv_ds) : 0.f;  // dL/dnu (and dL/dnu_t)
    if (PW) lphi += lnu * a.kvis;
    const float llap = -a.kf * phi * lA;
    lgsq -= a.kf6 * lA;
    lgr[0] += 2.f * gr[0] * lgsq;
    lgr[1] += 2.f * gr[1] * lgsq;
    lgr[2] += 2.f * gr[2] * lgsq;
    if (active) {
        a.aux[s] = lphi;
        a.aux[N + s] = llap;
        a.aux[2 * N + s] = lgr[0];
        a.aux[3 * N + s] = lgr[1];
        a.aux[4 * N + s] = lgr[2];
        a.aux[5 * N + s] = lp;
        a.aux[6 * N + s] = lu[0];
        a.aux[7 * N + s] = lu[1];
        a.aux[8 * N + s] = lu[2];
        if (LES) {
            // dwg/dnu_t = -3 wg^2 / ds, dnu_t/dtt = csd / (2 sqrt(tt)), dtt/dG_ab = 4 S_ab
            const float ltt = (les && tt > 0.f) ? lnu * (0.5f * a.csd / sqrtf(tt)) : 0.f;
#pragma unroll
            for (int al = 0; al < 3; ++al)
#pragma unroll
                for (int be = 0; be < 3; ++be)
                    a.aux[(size_t)(9 + al + 3 * be) * N + s] = ltt * 2.f * (G[al][be] + G[be][al]);
        }
        if (PW) a.aux[(size_t)18 * N + s] = wg;
        if (SPEC) {
            a.aux[(size_t)19 * N + s] = lF[0];
            a.aux[(size_t)20 * N + s] = lF[1];
            a.aux[(size_t)21 * N + s] = lF[2];
        }
    } else {
        dkf = dkg = domf = 0.f;
    }
    double gv[3] = {(double)dkf, (double)dkg, (double)domf};
    block_add<3>(gv, a.grads + 4 * (blockIdx.x % ADJ_NREP));
}

// lphi(x) = lphi_loc(x) - 14 llap(x)/5 + sum_k [llap(x - c_k)/5 + c_k . lgrad(x - c_k)/10],
// then the moments, plus the streamed (1 - w) part gathered from lin; writes
// lout (and lphi into phi_out for the initial state)
template <bool PW, bool LES>
__global__ void __launch_bounds__(256) adj_stencil(AdjArgs a, float* phi_out) {
    const long long s0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s0 >= (long long)a.N) return;
    const unsigned s = (unsigned)s0, N = a.N;
    const int x = (int)(s % a.nx), y = (int)((s / a.nx) % a.ny), z = (int)(s / ((unsigned)a.nx * a.ny));
    float lphi = a.aux[s] - 14.f * a.inv_lap * a.aux[N + s];
#pragma unroll
    for (int k = 1; k < Q; ++k) {
        const unsigned m = nbr(a, x, y, z, -cx(k), -cy(k), -cz(k));
        lphi += a.inv_lap * a.aux[N + m] +
                a.inv_grad * (cx(k) * a.aux[2 * N + m] + cy(k) * a.aux[3 * N + m] + cz(k) * a.aux[4 * N + m]);
    }
    const float lp = a.aux[5 * N + s] * (1.f / 3.f);
    float lu1 = a.aux[6 * N + s], lu2 = a.aux[7 * N + s], lu3 = a.aux[8 * N + s];
    float wg = a.stream ? a.omg : 1.f;
    if (LES && a.stream) {
        // transpose of G_ab(y) = inv_grad sum_k c_kb u_a(y + c_k): u_a(x) receives
        // inv_grad c_kb dL/dG_ab(x - c_k)
        float t[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 1; k < Q; ++k) {
            const unsigned m = nbr(a, x, y, z, -cx(k), -cy(k), -cz(k));
#pragma unroll
            for (int al = 0; al < 3; ++al) {
                float v = 0.f;
                if (cx(k)) v += cx(k) * a.aux[(size_t)(9 + al) * N + m];
                if (cy(k)) v += cy(k) * a.aux[(size_t)(9 + al + 3) * N + m];
                if (cz(k)) v += cz(k) * a.aux[(size_t)(9 + al + 6) * N + m];
                t[al] += v;
            }
        }
        lu1 += a.inv_grad * t[0];
        lu2 += a.inv_grad * t[1];
        lu3 += a.inv_grad * t[2];
    }
    if (PW && a.stream) wg = a.aux[(size_t)18 * N + s];
    if (phi_out) phi_out[s] = lphi;
    // the streamed part (1 - w) of the collision, gathered here rather than
    // stored by adj_local and read back
    const float wf = a.stream ? a.omf : 1.f;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const unsigned src = a.stream ? nbr(a, x, y, z, cx(i), cy(i), cz(i)) : s;
        a.lout[(size_t)i * N + s] = (1.f - wf) * a.lin[(size_t)i * N + src] + lphi;
        a.lout[(size_t)(Q + i) * N + s] =
            (1.f - wg) * a.lin[(size_t)(Q + i) * N + src] + (lp + (cx(i) * lu1 + cy(i) * lu2 + cz(i) * lu3));
    }
}

__global__ void adj_seed(const float* lphi, float* lam, unsigned N) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= (long long)N) return;
    const float v = lphi[s];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        lam[(size_t)i * N + s] = v;
        lam[(size_t)(Q + i) * N + s] = 0.f;
    }
}

static void fill_adj(dl_handle* h, AdjArgs& a) {
    const dl_params& P = h->P;
    memset(&a, 0, sizeof(a));
    a.nx = h->nx;
    a.ny = h->ny;
    a.nz = h->nz;
    a.N = (unsigned)h->N;
    a.phi1 = (float)P.phi1;
    a.omf = (float)(1.0 / P.tauf);
    a.omg = (float)(1.0 / (0.5 + 3.0 * P.nu1 / P.ds + (2.0 / 3.0) * P.Anu));
    a.kf = (float)P.kappaf;
    a.kf6 = (float)(P.kappaf / 6.0);
    a.kg = (float)P.kappag;
    a.T = (float)P.T;
    a.a = (float)P.a;
    a.b = (float)P.b;
    a.inv_lap = (float)(1.0 / (5.0 * P.ds * P.ds));
    a.inv_grad = (float)(1.0 / (10.0 * P.ds));
    const int bj[5] = {6, 11, 12, 13, 10}, tj[5] = {3, 14, 7, 8, 9};
    for (int k = 0; k < 5; ++k) {
        a.wbot[k] = (float)(6.0 * h->lc.E[bj[k]] * cx(bj[k]));   // g'_i = g'_j + 6 E_j U c_jx
        a.wtop[k] = (float)(-6.0 * h->lc.E[tj[k]] * cx(tj[k]));  // g'_i = g'_j - 6 E_j U c_jx
    }
    a.grads = h->adj_grads;
    a.aux = h->adj_aux;
    a.les = P.les ? 1 : 0;
    a.kvis = (float)((P.nu2 - P.nu1) / (P.phi2 - P.phi1));
    a.spec = h->force_mode == DL_FORCE_SPECTRAL ? 1 : 0;
    a.csd = (float)(P.Cs * P.Cs * P.delta * P.delta);
    a.nu1 = (float)P.nu1;
    a.inv_ds = (float)(1.0 / P.ds);
}

int adjoint_check(dl_handle* h) {
    if (h->form != DL_FORM_FP32 || h->single)
        return set_error(h, DL_ERR_UNSUPPORTED, "the adjoint is implemented for the two-phase FP32 form");
    if (h->P.les && h->P.Anu != 0.0) return set_error(h, DL_ERR_UNSUPPORTED, "the adjoint assumes A_nu = 0");
    if (h->P.nu2 != h->P.nu1 && h->P.visc_mode != DL_VISC_FIXED)
        return set_error(h, DL_ERR_UNSUPPORTED,
                         "a viscosity ratio other than 1 needs the fixed-range mode (the global phi range has no "
                         "adjoint here)");
    if (h->force_mode == DL_FORCE_SPECTRAL && h->sp.K < 1)
        return set_error(h, DL_ERR_UNSUPPORTED, "the adjoint of the spectral force needs the band plan");
    if (h->P.wall_u[1] != 0.0 || h->P.wall_u[2] != 0.0)
        return set_error(h, DL_ERR_UNSUPPORTED, "the adjoint assumes an x wall velocity");
    if (!h->adj_lam[0]) {
        for (int k = 0; k < 2; ++k) DL_CUDA(h, cudaMalloc(&h->adj_lam[k], sizeof(float) * 30 * h->N));
        DL_CUDA(h, cudaMalloc(&h->adj_aux, sizeof(float) * ADJ_AUX * h->N));
        DL_CUDA(h, cudaMalloc(&h->adj_grads, sizeof(double) * 4 * ADJ_NREP));
    }
    return DL_OK;
}

void adjoint_free(dl_handle* h) {
    for (int k = 0; k < 2; ++k) {
        cudaFree(h->adj_lam[k]);
        h->adj_lam[k] = nullptr;
    }
    cudaFree(h->adj_aux);
    cudaFree(h->adj_grads);
    h->adj_aux = nullptr;
    h->adj_grads = nullptr;
}

static inline unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

int adjoint_begin(dl_handle* h, const float* d_lphi) {
    int rc = adjoint_check(h);
    if (rc != DL_OK) return rc;
    DL_CUDA(h, cudaMemsetAsync(h->adj_grads, 0, sizeof(double) * 4 * ADJ_NREP, h->stream));
    h->adj_cur = 0;
    DL_LAUNCH(h, false, (adj_seed<<<nb(h->N), 256, 0, h->stream>>>(d_lphi, h->adj_lam[0], (unsigned)h->N)));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int adjoint_step(dl_handle* h, const float* d_state, long long step) {
    int rc = adjoint_check(h);
    if (rc != DL_OK) return rc;
    AdjArgs a;
    fill_adj(h, a);
    a.st = d_state;                           // adjoint state: f[15N], fields[5N] (, g[15N])
    a.mac = d_state + (size_t)Q * h->N;
    a.gst = d_state + (size_t)20 * h->N;
    a.lin = h->adj_lam[h->adj_cur];
    a.lout = h->adj_lam[1 - h->adj_cur];
    a.stream = 1;
    a.walls_on = (h->P.walls && step >= h->P.wall_start) ? 1 : 0;
    if (h->P.walls) {
        // the walls act on the adjoint of g' in place before the gather
        AdjArgs w = a;
        w.lout = h->adj_lam[h->adj_cur];
        w.walls_on = a.walls_on || h->P.walls;  // reflection happens even for a resting wall
        const long long plane = (long long)h->nx * h->ny;
        if (!a.walls_on)
            for (int k = 0; k < 5; ++k) w.wbot[k] = w.wtop[k] = 0.f;
        DL_LAUNCH(h, false, (adj_walls<<<nb(2 * plane), 256, 0, h->stream>>>(w)));
    }
    const bool pw = a.les || a.kvis != 0.f;
    const unsigned g = nb(h->N);
    cudaStream_t st = h->stream;
    if (!pw && !a.spec) DL_LAUNCH(h, true, (adj_local<false, false, false><<<g, 256, 0, st>>>(a)));
    else if (!pw) DL_LAUNCH(h, true, (adj_local<false, false, true><<<g, 256, 0, st>>>(a)));
    else if (!a.les && !a.spec) DL_LAUNCH(h, true, (adj_local<true, false, false><<<g, 256, 0, st>>>(a)));
    else if (!a.les) DL_LAUNCH(h, true, (adj_local<true, false, true><<<g, 256, 0, st>>>(a)));
    else if (!a.spec) DL_LAUNCH(h, true, (adj_local<true, true, false><<<g, 256, 0, st>>>(a)));
    else DL_LAUNCH(h, true, (adj_local<true, true, true><<<g, 256, 0, st>>>(a)));
    if (a.spec) {
        const size_t N = h->N;
        float* x = h->adj_aux;
        const float* m = a.mac;
        rc = spectral_adjoint_f32(h, x + 19 * N, x + 20 * N, x + 21 * N, m + N, m + 2 * N, m + 3 * N, x + 6 * N,
                                  x + 7 * N, x + 8 * N);
        if (rc != DL_OK) return rc;
    }
    if (!pw) DL_LAUNCH(h, false, (adj_stencil<false, false><<<g, 256, 0, st>>>(a, nullptr)));
    else if (!a.les) DL_LAUNCH(h, false, (adj_stencil<true, false><<<g, 256, 0, st>>>(a, nullptr)));
    else DL_LAUNCH(h, false, (adj_stencil<true, true><<<g, 256, 0, st>>>(a, nullptr)));
    DL_CUDA(h, cudaGetLastError());
    h->adj_cur = 1 - h->adj_cur;
    return DL_OK;
}

int adjoint_init(dl_handle* h, const float* d_state0, float* d_lphi0) {
    int rc = adjoint_check(h);
    if (rc != DL_OK) return rc;
    AdjArgs a;
    fill_adj(h, a);
    a.st = d_state0;                          // full state: f[15N], g[15N], fields[5N]
    a.mac = d_state0 + (size_t)30 * h->N;
    a.lin = h->adj_lam[h->adj_cur];
    a.lout = h->adj_lam[1 - h->adj_cur];
    a.stream = 0;
    DL_LAUNCH(h, false, (adj_local<false, false, false><<<nb(h->N), 256, 0, h->stream>>>(a)));
    DL_LAUNCH(h, false, (adj_stencil<false, false><<<nb(h->N), 256, 0, h->stream>>>(a, d_lphi0)));
    DL_CUDA(h, cudaGetLastError());
    h->adj_cur = 1 - h->adj_cur;
    return DL_OK;
}

int adjoint_grads(dl_handle* h, double* out4) {
    if (!h->adj_grads) return set_error(h, DL_ERR_STATE, "no adjoint pass has run");
    double rep[4 * ADJ_NREP];
    DL_CUDA(h, cudaMemcpyAsync(rep, h->adj_grads, sizeof(rep), cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 4; ++k) {
        double s = 0.0;
        for (int r = 0; r < ADJ_NREP; ++r) s += rep[4 * r + k];
        out4[k] = s;
    }
    // d/dtau_f = d/domega_f * d omega_f / d tau_f = -d/domega_f / tau_f^2
    out4[2] = -out4[2] / (h->P.tauf * h->P.tauf);
    return DL_OK;
}

}  // namespace dl
