// spectral.cu -- constant-injection band forcing of the forced-turbulence
// droplet code, externalforce in program/lbm_drop_iht_xy.f90:722-842:
//   u_hat = FFT(u) / N                        (fft_r2c, :894-901)
//   E     = sum_{half spectrum, 1 <= |k| < kc} 0.5 |u_hat|^2 min(2, k3+1)   (:775-795)
//   f_hat = (0.5 eps / E) u_hat on the band, 0 elsewhere                   (:797-818)
//   F     = c2r(f_hat), not normalised         (fft_c2r, :903-908)
// Only the band modes are non-zero, so instead of six full 3-D FFTs per step
// the transform is an exact separable DFT over the 2K+1 (K = kc-1) wavenumbers
// per axis that the band can touch: an x stage over every (y, z) row, then y,
// then z, and the mirror-image synthesis. In the FP64 form every sum runs in
// the same sequential order as the oracle's restatement, so both give the
// same bits; they differ from an FFT by rounding only.
#include "dl_internal.cuh"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

namespace dl {

struct SpArgs {
    int nx, ny, nz, K, kc2;
    const double* u[3];
    double* fo[3];
    const double* twx;
    const double* twy;
    const double* twz;
    double* a1;  // [3][NK][ny][nz] complex -> index ((c*NK + kx)*ny + y)*nz + z
    double* a2;  // [3][NK][NK][nz]
    double* uh;  // [3][NK][NK][K+1]
    double* b1;  // [3][NK][NK][nz]
    double* b2;  // [3][NK][ny][nz]
    DevState* st;
    double half_eps;
    double Nd;
};

__device__ __forceinline__ int modi(long long v, int n) { return (int)(((v % n) + n) % n); }

// x stage: a1[c][kx][y][z] = sum_x u e^{-i 2 pi kx x / nx}
__global__ void sp_xstage(const SpArgs a) {
    const int NK = 2 * a.K + 1;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = 3LL * NK * a.ny * a.nz;
    if (t >= total) return;
    const int z = (int)(t % a.nz);
    long long r = t / a.nz;
    const int y = (int)(r % a.ny);
    r /= a.ny;
    const int kxi = (int)(r % NK);
    const int c = (int)(r / NK);
    const int kx = kxi - a.K;
    const double* u = a.u[c] + ((long long)z * a.ny + y) * a.nx;
    double re = 0.0, im = 0.0;
    for (int x = 0; x < a.nx; ++x) {
        const int m = modi((long long)kx * x, a.nx);
        const double v = u[x];
        re = re + v * a.twx[2 * m];
        im = im - v * a.twx[2 * m + 1];
    }
    double* d = a.a1 + 2 * ((((long long)c * NK + kxi) * a.ny + y) * a.nz + z);
    d[0] = re;
    d[1] = im;
}

// y stage: a2[c][kx][ky][z] = sum_y a1 e^{-i 2 pi ky y / ny}
__global__ void sp_ystage(const SpArgs a) {
    const int NK = 2 * a.K + 1;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = 3LL * NK * NK * a.nz;
    if (t >= total) return;
    const int z = (int)(t % a.nz);
    long long r = t / a.nz;
    const int kyi = (int)(r % NK);
    r /= NK;
    const int kxi = (int)(r % NK);
    const int c = (int)(r / NK);
    const int ky = kyi - a.K;
    double re = 0.0, im = 0.0;
    for (int y = 0; y < a.ny; ++y) {
        const int m = modi((long long)ky * y, a.ny);
        const double* v = a.a1 + 2 * ((((long long)c * NK + kxi) * a.ny + y) * a.nz + z);
        const double cy_ = a.twy[2 * m], sy_ = a.twy[2 * m + 1];
        re = re + (v[0] * cy_ + v[1] * sy_);
        im = im + (v[1] * cy_ - v[0] * sy_);
    }
    double* d = a.a2 + 2 * ((((long long)c * NK + kxi) * NK + kyi) * a.nz + z);
    d[0] = re;
    d[1] = im;
}

// z stage: uh[c][kx][ky][kz] = (sum_z a2 e^{-i 2 pi kz z / nz}) / N, kz = 0..K
__global__ void sp_zstage(const SpArgs a) {
    const int NK = 2 * a.K + 1;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = 3LL * NK * NK * (a.K + 1);
    if (t >= total) return;
    const int kz = (int)(t % (a.K + 1));
    long long r = t / (a.K + 1);
    const int kyi = (int)(r % NK);
    r /= NK;
    const int kxi = (int)(r % NK);
    const int c = (int)(r / NK);
    double re = 0.0, im = 0.0;
    for (int z = 0; z < a.nz; ++z) {
        const int m = (int)(((long long)kz * z) % a.nz);
        const double* v = a.a2 + 2 * ((((long long)c * NK + kxi) * NK + kyi) * a.nz + z);
        const double cz_ = a.twz[2 * m], sz_ = a.twz[2 * m + 1];
        re = re + (v[0] * cz_ + v[1] * sz_);
        im = im + (v[1] * cz_ - v[0] * sz_);
    }
    double* d = a.uh + 2 * ((((long long)c * NK + kxi) * NK + kyi) * (a.K + 1) + kz);
    d[0] = re / a.Nd;
    d[1] = im / a.Nd;
}

// band energy in the reference's loop order (k3 outer, then k2, then k1, each
// in FFT index order) and the coefficient 0.5 eps / E; one thread.
__global__ void sp_energy(const SpArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int NK = 2 * a.K + 1;
    double energy = 0.0;
    for (int k3 = 0; k3 <= a.K; ++k3)
        for (int i2 = 0; i2 < a.ny; ++i2) {
            const int k2 = (i2 >= a.ny / 2 + 1) ? i2 - a.ny : i2;
            if (k2 < -a.K || k2 > a.K) continue;
            for (int i1 = 0; i1 < a.nx; ++i1) {
                const int k1 = (i1 >= a.nx / 2 + 1) ? i1 - a.nx : i1;
                if (k1 < -a.K || k1 > a.K) continue;
                const int kk = k1 * k1 + k2 * k2 + k3 * k3;
                if (kk < 1 || kk >= a.kc2) continue;
                double e[3];
                for (int c = 0; c < 3; ++c) {
                    const double* v = a.uh + 2 * ((((long long)c * NK + (k1 + a.K)) * NK + (k2 + a.K)) * (a.K + 1) + k3);
                    e[c] = v[0] * v[0] + v[1] * v[1];
                }
                const double w = 2.0 < (double)k3 + 1.0 ? 2.0 : (double)k3 + 1.0;
                energy = energy + 0.5 * (e[0] + e[1] + e[2]) * w;
            }
        }
    a.st->sp_energy = energy;
    a.st->sp_coef = a.half_eps / energy;
}

// synthesis, kz then ky then kx, as the c2r of the half spectrum:
// F = sum_kz w(kz) Re(sum f_hat e^{+ik.x}), w = 1 for kz = 0 and 2 otherwise
__global__ void sp_synth_z(const SpArgs a) {
    const int NK = 2 * a.K + 1;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = 3LL * NK * NK * a.nz;
    if (t >= total) return;
    const int z = (int)(t % a.nz);
    long long r = t / a.nz;
    const int kyi = (int)(r % NK);
    r /= NK;
    const int kxi = (int)(r % NK);
    const int c = (int)(r / NK);
    const int kx = kxi - a.K, ky = kyi - a.K;
    const double coef = a.st->sp_coef;
    double re = 0.0, im = 0.0;
    for (int kz = 0; kz <= a.K; ++kz) {
        const int kk = kx * kx + ky * ky + kz * kz;
        if (kk < 1 || kk >= a.kc2) continue;
        const double* v = a.uh + 2 * ((((long long)c * NK + kxi) * NK + kyi) * (a.K + 1) + kz);
        const double fre = coef * v[0], fim = coef * v[1];
        const double w = kz == 0 ? 1.0 : 2.0;
        const int m = (int)(((long long)kz * z) % a.nz);
        const double cz_ = a.twz[2 * m], sz_ = a.twz[2 * m + 1];
        re = re + w * (fre * cz_ - fim * sz_);
        im = im + w * (fre * sz_ + fim * cz_);
    }
    double* d = a.b1 + 2 * ((((long long)c * NK + kxi) * NK + kyi) * a.nz + z);
    d[0] = re;
    d[1] = im;
}

__global__ void sp_synth_y(const SpArgs a) {
    const int NK = 2 * a.K + 1;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = 3LL * NK * a.ny * a.nz;
    if (t >= total) return;
    const int z = (int)(t % a.nz);
    long long r = t / a.nz;
    const int y = (int)(r % a.ny);
    r /= a.ny;
    const int kxi = (int)(r % NK);
    const int c = (int)(r / NK);
    double re = 0.0, im = 0.0;
    for (int kyi = 0; kyi < NK; ++kyi) {
        const int ky = kyi - a.K;
        const double* v = a.b1 + 2 * ((((long long)c * NK + kxi) * NK + kyi) * a.nz + z);
        const int m = modi((long long)ky * y, a.ny);
        const double cy_ = a.twy[2 * m], sy_ = a.twy[2 * m + 1];
        re = re + (v[0] * cy_ - v[1] * sy_);
        im = im + (v[0] * sy_ + v[1] * cy_);
    }
    double* d = a.b2 + 2 * ((((long long)c * NK + kxi) * a.ny + y) * a.nz + z);
    d[0] = re;
    d[1] = im;
}

__global__ void sp_synth_x(const SpArgs a) {
    const int NK = 2 * a.K + 1;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long N = (long long)a.nx * a.ny * a.nz;
    if (t >= 3 * N) return;
    const int c = (int)(t / N);
    const long long s = t - c * N;
    const int x = (int)(s % a.nx);
    const long long r = s / a.nx;
    const int y = (int)(r % a.ny);
    const int z = (int)(r / a.ny);
    double re = 0.0;
    for (int kxi = 0; kxi < NK; ++kxi) {
        const int kx = kxi - a.K;
        const double* v = a.b2 + 2 * ((((long long)c * NK + kxi) * a.ny + y) * a.nz + z);
        const int m = modi((long long)kx * x, a.nx);
        re = re + (v[0] * a.twx[2 * m] - v[1] * a.twx[2 * m + 1]);
    }
    a.fo[c][s] = re;
}

// FP32 forms: the x stage with one warp per (y, z) row (lanes over x, FP32
// sums, reduced across the warp), and the x synthesis writing FP32 forces.
// The small y / z stages and the energy are shared with the FP64 form.
constexpr int SP_KMAX = 4;  // supports kc <= 5

__global__ void sp_xstage_f32(const float* __restrict__ u1, const float* __restrict__ u2,
                              const float* __restrict__ u3, double* __restrict__ a1, int nx, int ny, int nz, int K,
                              const float* __restrict__ tw) {
    const int lane = threadIdx.x & 31;
    const long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    if (row >= (long long)ny * nz) return;
    const int z = (int)(row / ny), y = (int)(row - (long long)z * ny);
    const int NK = 2 * K + 1;
    const float* u[3] = {u1, u2, u3};
    const long long base = ((long long)z * ny + y) * nx;
    float re[3][2 * SP_KMAX + 1], im[3][2 * SP_KMAX + 1];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < NK; ++k) re[c][k] = im[c][k] = 0.f;
    for (int x = lane; x < nx; x += 32) {
        const float v[3] = {u[0][base + x], u[1][base + x], u[2][base + x]};
        for (int k = 0; k < NK; ++k) {
            int m = ((k - K) * x) % nx;
            m = m < 0 ? m + nx : m;
            const float cs = tw[2 * m], sn = tw[2 * m + 1];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                re[c][k] += v[c] * cs;
                im[c][k] -= v[c] * sn;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < NK; ++k) {
            float r = re[c][k], i = im[c][k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                r += __shfl_xor_sync(0xffffffffu, r, o);
                i += __shfl_xor_sync(0xffffffffu, i, o);
            }
            if (lane == 0) {
                double* d = a1 + 2 * ((((long long)c * NK + k) * ny + y) * nz + z);
                d[0] = (double)r;
                d[1] = (double)i;
            }
        }
}

__global__ void sp_synth_x_f32(const double* __restrict__ b2, float* __restrict__ fx, float* __restrict__ fy,
                               float* __restrict__ fz, int nx, int ny, int nz, int K, const float* __restrict__ tw) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long N = (long long)nx * ny * nz;
    if (s >= N) return;
    const int x = (int)(s % nx);
    const long long r = s / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const int NK = 2 * K + 1;
    float out[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < NK; ++k) {
        int m = ((k - K) * x) % nx;
        m = m < 0 ? m + nx : m;
        const float cs = tw[2 * m], sn = tw[2 * m + 1];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double* v = b2 + 2 * ((((long long)c * NK + k) * ny + y) * nz + z);
            out[c] += (float)v[0] * cs - (float)v[1] * sn;
        }
    }
    fx[s] = out[0];
    fy[s] = out[1];
    fz[s] = out[2];
}

// ---- adjoint of the band force (reverse pass of a step with the spectral force) ----
// F = coef v with v = P u, the band-pass of u (sum over the band of w Re(u_hat
// e^{ik.x}), u_hat = DFT(u)/N), coef = 0.5 eps / E and E = sum w 0.5 |u_hat|^2 =
// |v|^2 / 2N. For lF = dL/dF, since P is a symmetric projection and dE/du = v/N:
//   dL/du = coef P lF - (s coef / (E N)) v,   s = sum_x lF . v = N sum w Re(u_hat conj(L_hat)),
// with L_hat the band coefficients of lF: one synthesis of the combined
// coefficients coef L_hat - (s coef / (E N)) u_hat. One block; reads E and coef
// that sp_energy left, writes the combination into uh and sets coef = 1 for
// the synthesis kernels.
__global__ void sp_adj_combine(const SpArgs a, const double* __restrict__ lh) {
    __shared__ double s_part[32];
    const int NK = 2 * a.K + 1;
    const int nv = 3 * NK * NK * (a.K + 1);
    const double E = a.st->sp_energy, coef = a.st->sp_coef;
    double s = 0.0;
    for (int t = threadIdx.x; t < nv; t += blockDim.x) {
        const int kz = t % (a.K + 1), r = t / (a.K + 1), kyi = r % NK, kxi = (r / NK) % NK;
        const int kx = kxi - a.K, ky = kyi - a.K, kk = kx * kx + ky * ky + kz * kz;
        if (kk < 1 || kk >= a.kc2) continue;
        const double w = kz == 0 ? 1.0 : 2.0;
        s += w * (a.uh[2 * t] * lh[2 * t] + a.uh[2 * t + 1] * lh[2 * t + 1]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = s;
    __syncthreads();
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s_part[w];
    const double g = tot * coef / E;  // s coef / (E N), s = N tot
    for (int t = threadIdx.x; t < 2 * nv; t += blockDim.x) a.uh[t] = coef * lh[t] - g * a.uh[t];
    __syncthreads();
    if (threadIdx.x == 0) a.st->sp_coef = 1.0;
}

// the x synthesis added into FP32 arrays
__global__ void sp_synth_x_add_f32(const double* __restrict__ b2, float* __restrict__ o1, float* __restrict__ o2,
                                   float* __restrict__ o3, int nx, int ny, int nz, int K,
                                   const float* __restrict__ tw) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long N = (long long)nx * ny * nz;
    if (s >= N) return;
    const int x = (int)(s % nx);
    const long long r = s / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const int NK = 2 * K + 1;
    float out[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < NK; ++k) {
        int m = ((k - K) * x) % nx;
        m = m < 0 ? m + nx : m;
        const float cs = tw[2 * m], sn = tw[2 * m + 1];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double* v = b2 + 2 * ((((long long)c * NK + k) * ny + y) * nz + z);
            out[c] += (float)v[0] * cs - (float)v[1] * sn;
        }
    }
    o1[s] += out[0];
    o2[s] += out[1];
    o3[s] += out[2];
}

static int upload_twiddle(dl_handle* h, int n, double** d) {
    std::vector<double> t(2 * (size_t)n);
    const double pi = acos(-1.0);
    for (int m = 0; m < n; ++m) {
        const double ang = 2.0 * pi * (double)m / (double)n;
        t[2 * m] = cos(ang);
        t[2 * m + 1] = sin(ang);
    }
    DL_CUDA(h, cudaMalloc(d, sizeof(double) * 2 * n));
    DL_CUDA(h, cudaMemcpy(*d, t.data(), sizeof(double) * 2 * n, cudaMemcpyHostToDevice));
    return DL_OK;
}

int spectral_alloc(dl_handle* h) {
    SpectralPlan& sp = h->sp;
    memset(&sp, 0, sizeof(sp));
    const int K = h->P.kc - 1;
    sp.K = K;
    if (K < 1) return DL_OK;
    if (2 * K + 1 > h->nx || 2 * K + 1 > h->ny || K + 1 > h->nz / 2) {
        // no band plan: dl_set_force(DL_FORCE_SPECTRAL) refuses; the step itself works
        sp.K = 0;
        return DL_OK;
    }
    const int NK = 2 * K + 1;
    int rc;
    if ((rc = upload_twiddle(h, h->nx, &sp.d_twx)) != DL_OK) return rc;
    if ((rc = upload_twiddle(h, h->ny, &sp.d_twy)) != DL_OK) return rc;
    if ((rc = upload_twiddle(h, h->nz, &sp.d_twz)) != DL_OK) return rc;
    if (K > SP_KMAX) return set_error(h, DL_ERR_ARG, "kc=%d above the supported maximum %d", h->P.kc, SP_KMAX + 1);
    {
        std::vector<float> t(2 * (size_t)h->nx);
        const double pi = acos(-1.0);
        for (int m = 0; m < h->nx; ++m) {
            t[2 * m] = (float)cos(2.0 * pi * m / h->nx);
            t[2 * m + 1] = (float)sin(2.0 * pi * m / h->nx);
        }
        DL_CUDA(h, cudaMalloc(&sp.d_twxf, sizeof(float) * 2 * h->nx));
        DL_CUDA(h, cudaMemcpy(sp.d_twxf, t.data(), sizeof(float) * 2 * h->nx, cudaMemcpyHostToDevice));
    }
    const size_t rows = (size_t)h->ny * h->nz;
    DL_CUDA(h, cudaMalloc(&sp.d_a1, sizeof(double) * 2 * 3 * NK * rows));
    DL_CUDA(h, cudaMalloc(&sp.d_b2, sizeof(double) * 2 * 3 * NK * rows));
    // a2 and b1 share one buffer: [3][NK][NK][nz] complex each
    DL_CUDA(h, cudaMalloc(&sp.d_uh, sizeof(double) * 2 * 3 * NK * NK * ((size_t)K + 1 + 2 * (size_t)h->nz)));
    int nm = 0;
    for (int kz = 0; kz <= K; ++kz)
        for (int ky = -K; ky <= K; ++ky)
            for (int kx = -K; kx <= K; ++kx) {
                int kk = kx * kx + ky * ky + kz * kz;
                if (kk >= 1 && kk < h->P.kc * h->P.kc) ++nm;
            }
    sp.nmodes = nm;
    return DL_OK;
}

void spectral_free(dl_handle* h) {
    SpectralPlan& sp = h->sp;
    cudaFree(sp.d_twx);
    cudaFree(sp.d_twy);
    cudaFree(sp.d_twz);
    cudaFree(sp.d_a1);
    cudaFree(sp.d_b2);
    cudaFree(sp.d_uh);
    cudaFree(sp.d_twxf);
    cudaFree(sp.d_lh);
    memset(&sp, 0, sizeof(sp));
}

static void fill_sp(dl_handle* h, SpArgs& a) {
    memset(&a, 0, sizeof(a));
    const SpectralPlan& sp = h->sp;
    const int NK = 2 * sp.K + 1;
    a.nx = h->nx;
    a.ny = h->ny;
    a.nz = h->nz;
    a.K = sp.K;
    a.kc2 = h->P.kc * h->P.kc;
    a.twx = sp.d_twx;
    a.twy = sp.d_twy;
    a.twz = sp.d_twz;
    a.a1 = sp.d_a1;
    a.b2 = sp.d_b2;
    a.uh = sp.d_uh;
    a.a2 = sp.d_uh + 2 * 3 * NK * NK * (size_t)(sp.K + 1);
    a.b1 = a.a2 + 2 * 3 * NK * NK * (size_t)h->nz;
    a.st = h->d_state;
    a.half_eps = 0.5 * h->P.eps;
    a.Nd = (double)h->nx * (double)h->ny * (double)h->nz;
}

static inline unsigned nb(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int spectral_force_fp64(dl_handle* h, const double* u1, const double* u2, const double* u3, double* fx,
                        double* fy, double* fz) {
    SpArgs a;
    fill_sp(h, a);
    a.u[0] = u1;
    a.u[1] = u2;
    a.u[2] = u3;
    a.fo[0] = fx;
    a.fo[1] = fy;
    a.fo[2] = fz;
    const int NK = 2 * a.K + 1;
    const long long N = (long long)h->N;
    cudaStream_t s = h->stream;
    DL_LAUNCH(h, false, sp_xstage<<<nb(3LL * NK * h->ny * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_ystage<<<nb(3LL * NK * NK * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_zstage<<<nb(3LL * NK * NK * (a.K + 1), 64), 64, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_energy<<<1, 32, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_z<<<nb(3LL * NK * NK * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_y<<<nb(3LL * NK * h->ny * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_x<<<nb(3 * N, 256), 256, 0, s>>>(a));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

// forward part only: sp.d_uh = band coefficients u_hat / N of an FP32 u
int spectral_project_f32(dl_handle* h, const float* u1, const float* u2, const float* u3) {
    SpArgs a;
    fill_sp(h, a);
    const int NK = 2 * a.K + 1;
    cudaStream_t s = h->stream;
    const long long rows = (long long)h->ny * h->nz;
    DL_LAUNCH(h, false, sp_xstage_f32<<<nb(rows * 32, 256), 256, 0, s>>>(u1, u2, u3, a.a1, h->nx, h->ny, h->nz, a.K,
                                                                        h->sp.d_twxf));
    DL_LAUNCH(h, false, sp_ystage<<<nb(3LL * NK * NK * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_zstage<<<nb(3LL * NK * NK * (a.K + 1), 64), 64, 0, s>>>(a));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

// dL/du of the band force added into lu, from dL/dF (lf) and the u the force was
// computed from
int spectral_adjoint_f32(dl_handle* h, const float* lf1, const float* lf2, const float* lf3, const float* u1,
                         const float* u2, const float* u3, float* lu1, float* lu2, float* lu3) {
    SpectralPlan& sp = h->sp;
    if (sp.K < 1) return set_error(h, DL_ERR_STATE, "no band plan for the spectral force");
    const int NK = 2 * sp.K + 1;
    const size_t nuh = (size_t)2 * 3 * NK * NK * (sp.K + 1);
    if (!sp.d_lh) DL_CUDA(h, cudaMalloc(&sp.d_lh, sizeof(double) * nuh));
    int rc = spectral_project_f32(h, lf1, lf2, lf3);
    if (rc != DL_OK) return rc;
    DL_CUDA(h, cudaMemcpyAsync(sp.d_lh, sp.d_uh, sizeof(double) * nuh, cudaMemcpyDeviceToDevice, h->stream));
    rc = spectral_project_f32(h, u1, u2, u3);
    if (rc != DL_OK) return rc;
    SpArgs a;
    fill_sp(h, a);
    cudaStream_t s = h->stream;
    const long long N = (long long)h->N;
    DL_LAUNCH(h, false, sp_energy<<<1, 32, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_adj_combine<<<1, 256, 0, s>>>(a, sp.d_lh));
    DL_LAUNCH(h, false, sp_synth_z<<<nb(3LL * NK * NK * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_y<<<nb(3LL * NK * h->ny * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_x_add_f32<<<nb(N, 256), 256, 0, s>>>(a.b2, lu1, lu2, lu3, h->nx, h->ny, h->nz, a.K,
                                                                       sp.d_twxf));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int spectral_force_f32(dl_handle* h, const float* u1, const float* u2, const float* u3, float* fx, float* fy,
                       float* fz) {
    SpArgs a;
    fill_sp(h, a);
    const int NK = 2 * a.K + 1;
    const long long N = (long long)h->N;
    cudaStream_t s = h->stream;
    const long long rows = (long long)h->ny * h->nz;
    DL_LAUNCH(h, false, sp_xstage_f32<<<nb(rows * 32, 256), 256, 0, s>>>(u1, u2, u3, a.a1, h->nx, h->ny, h->nz, a.K,
                                                                        h->sp.d_twxf));
    DL_LAUNCH(h, false, sp_ystage<<<nb(3LL * NK * NK * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_zstage<<<nb(3LL * NK * NK * (a.K + 1), 64), 64, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_energy<<<1, 32, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_z<<<nb(3LL * NK * NK * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_y<<<nb(3LL * NK * h->ny * h->nz, 128), 128, 0, s>>>(a));
    DL_LAUNCH(h, false, sp_synth_x_f32<<<nb(N, 256), 256, 0, s>>>(a.b2, fx, fy, fz, h->nx, h->ny, h->nz, a.K,
                                                                   h->sp.d_twxf));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

}  // namespace dl
