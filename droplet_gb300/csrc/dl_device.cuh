// dl_device.cuh -- device helpers shared by the step kernels of every form.
#pragma once

#include "dl_internal.cuh"

namespace dl {

__device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// Block-level min/max of phi, one atomic per block, and the last block's
// finalisation of the reference's serial scan (program/lbm_drop_xy.f90:559-571):
//   max = phi1; min = phi2; for each phi in z,y,x order:
//       if (phi > max) max = phi; else if (phi < min) min = phi
// Its result equals max(phi1, max phi) and min(phi2, min phi) except when
// every phi exceeds phi1 and the first site holds the smallest value; that
// case is resolved by an exact ordered scan in the last block.
// phi values are phi_off + phi_new[k] evaluated in T (the FP32 forms store
// phi - phi1 and pass phi_off = phi1).
// nblk is the number of blocks that reduce into st (the whole grid for one
// domain). Returns true in the last block (after it has finalised).
template <typename T>
__device__ bool minmax_block_and_finalize(DevState* st, double vmin, double vmax, const T* phi_new, T phi_off,
                                          long long N, double phi1, double phi2, bool nan_seen,
                                          long long step, unsigned nblk) {
    __shared__ long long smin[32], smax[32];
    __shared__ int s_last;
    __shared__ int s_nan;
    long long kmin = dbl_key(vmin), kmax = dbl_key(vmax);
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_nan = 0;
    __syncthreads();
    if (nan_seen) s_nan = 1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long a = __shfl_xor_sync(0xffffffffu, kmin, o);
        long long b = __shfl_xor_sync(0xffffffffu, kmax, o);
        kmin = a < kmin ? a : kmin;
        kmax = b > kmax ? b : kmax;
    }
    if (lane == 0) {
        smin[warp] = kmin;
        smax[warp] = kmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int w = 1; w < nw; ++w) {
            kmin = smin[w] < kmin ? smin[w] : kmin;
            kmax = smax[w] > kmax ? smax[w] : kmax;
        }
        kmin = smin[0] < kmin ? smin[0] : kmin;
        kmax = smax[0] > kmax ? smax[0] : kmax;
        atomicMin(&st->key_min, kmin);
        atomicMax(&st->key_max, kmax);
        if (s_nan) {
            if (atomicExch(&st->nan_flag, 1) == 0) st->nan_step = step;
        }
        __threadfence();
        unsigned t = atomicAdd(&st->blocks_done, 1u);
        s_last = (t == nblk - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    // ---- last block: finalise ----
    __shared__ double s_mn, s_mx;
    __shared__ int s_rare;
    if (threadIdx.x == 0) {
        const long long K0 = atomicAdd((unsigned long long*)&st->key_min, 0ull);
        const long long K1 = atomicAdd((unsigned long long*)&st->key_max, 0ull);
        const double gmin = key_dbl(K0), gmax = key_dbl(K1);
        const double e1 = (double)(phi_off + __ldcg(phi_new));
        s_mx = (gmax > phi1) ? gmax : phi1;
        s_rare = (K0 != KEY_POS_INF) && (gmin > phi1) && (e1 == gmin);
        s_mn = (gmin < phi2) ? gmin : phi2;
    }
    __syncthreads();
    if (s_rare) {
        // exact ordered scan: phi_k counts for the minimum iff phi_k <= the
        // running maximum before it (seeded with phi1); NaN never counts.
        __shared__ double sm[32], sx[32];
        __shared__ double s_carry, s_cand;
        if (threadIdx.x == 0) {
            s_carry = phi1;
            s_cand = phi2;
        }
        __syncthreads();
        for (long long base = 0; base < N; base += blockDim.x) {
            long long k = base + threadIdx.x;
            double v = (k < N) ? (double)(phi_off + __ldcg(phi_new + k)) : -INFINITY;
            double sv = (v == v) ? v : -INFINITY;
            // inclusive block scan of max
            double incl = sv;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                double t = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl = fmax(incl, t);
            }
            if (lane == 31) sx[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                const int nw = (blockDim.x + 31) >> 5;
                double w = (lane < (unsigned)nw) ? sx[lane] : -INFINITY;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    double t = __shfl_up_sync(0xffffffffu, w, o);
                    if ((int)lane >= o) w = fmax(w, t);
                }
                if (lane < (unsigned)nw) sx[lane] = w;
            }
            __syncthreads();
            double prev_in_warp = __shfl_up_sync(0xffffffffu, incl, 1);
            double before = (lane == 0) ? -INFINITY : prev_in_warp;
            if (warp > 0) before = fmax(before, sx[warp - 1]);
            before = fmax(before, s_carry);
            double cand = (k < N && v == v && v <= before) ? v : INFINITY;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) cand = fmin(cand, __shfl_xor_sync(0xffffffffu, cand, o));
            if (lane == 0) sm[warp] = cand;
            __syncthreads();
            if (threadIdx.x == 0) {
                const int nw = (blockDim.x + 31) >> 5;
                double c = INFINITY;
                for (int w = 0; w < nw; ++w) c = fmin(c, sm[w]);
                if (c < s_cand) s_cand = c;
                s_carry = fmax(s_carry, sx[nw - 1]);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            s_mn = s_cand;
            st->quirk_scans += 1;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st->phi_min = s_mn;
        st->phi_max = s_mx;
        st->key_min = KEY_POS_INF;
        st->key_max = KEY_NEG_INF;
        __threadfence();
        st->blocks_done = 0u;
    }
    return true;
}

}  // namespace dl
