// dl_internal.cuh -- internal declarations shared by the translation units of
// libdroplet_gb300.so. Not part of the C-ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>

#include "../../include/droplet_gb300.h"

namespace dl {

// D3Q15 lattice (program/lbm_drop_xy.f90:70-84); directions 0..14 = reference 1..15.
constexpr int Q = 15;
__host__ __device__ constexpr int cx(int i) {
    return (i == 1 || i == 7 || i == 9 || i == 10 || i == 12) ? 1
         : (i == 4 || i == 8 || i == 11 || i == 13 || i == 14) ? -1 : 0;
}
__host__ __device__ constexpr int cy(int i) {
    return (i == 2 || i == 7 || i == 8 || i == 10 || i == 13) ? 1
         : (i == 5 || i == 9 || i == 11 || i == 12 || i == 14) ? -1 : 0;
}
__host__ __device__ constexpr int cz(int i) {
    return (i == 3 || i == 7 || i == 8 || i == 9 || i == 14) ? 1
         : (i == 6 || i == 10 || i == 11 || i == 12 || i == 13) ? -1 : 0;
}
// weight class: 0 rest, 1 axis, 2 body diagonal
__host__ __device__ constexpr int wclass(int i) { return i == 0 ? 0 : (i <= 6 ? 1 : 2); }

// Host-computed constants (double), in the reference's rounding: each entry is
// the correctly rounded value of the reference's constant expression.
struct LatticeConsts {
    double E[Q], F[Q];
    double Ekf[Q];     // E(i)*kappaf
    double Ekg[Q];     // E(i)*kappag
    double ds3E[Q];    // (3*ds)*E(i)
    double six_E[Q];   // 6*E(i)
};

// Device-resident per-handle state (scratch: reduction accumulators, flags).
struct DevState {
    double phi_min, phi_max;         // tau_g interpolation range of the next step
    long long key_min, key_max;      // ordered-integer min/max accumulators of this step
    unsigned int blocks_done;        // last-block ticket of the step kernel
    int nan_flag;                    // nonzero once a non-finite value was produced
    long long nan_step;              // step at which it was first seen
    int quirk_scans;                 // number of exact serial-order min scans taken
    int wait_timeout;                // nonzero once a bounded device-side wait ran out
    // spectral forcing
    double sp_energy;                // band energy of the last forcing evaluation
    double sp_coef;                  // 0.5 eps / E
    unsigned int sp_done;            // last-block ticket of the band projection
    unsigned int pad2_;
};

// Ordered mapping of a double to a signed 64-bit key (monotone for non-NaN).
__host__ __device__ inline long long dbl_key(double v) {
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(v);
#else
    long long b;
    memcpy(&b, &v, 8);
#endif
    return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}
__host__ __device__ inline double key_dbl(long long k) {
    long long b = k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFLL);
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double v;
    memcpy(&v, &b, 8);
    return v;
#endif
}
constexpr long long KEY_POS_INF = 0x7FF0000000000000LL;                  // key of +inf
constexpr long long KEY_NEG_INF = (long long)0xFFF0000000000000ULL ^ 0x7FFFFFFFFFFFFFFFLL;  // key of -inf

// Spectral forcing tables (band 1 <= |k| < kc, half spectrum kz >= 0).
struct SpectralPlan {
    int K;            // kc - 1
    int nmodes;       // number of half-spectrum band modes
    double* d_twx;    // [nx][2] cos, sin of 2 pi m / nx
    double* d_twy;    // [ny][2]
    double* d_twz;    // [nz][2]
    double* d_a1;     // [3][2K+1][ny*nz] complex   (x stage)
    double* d_uh;     // [3][2K+1][2K+1][K+1] complex (band coefficients, /N)
    double* d_b2;     // [3][2K+1][ny*nz] complex   (synthesis, x pending)
    float* d_twxf;    // FP32 copy of d_twx
    double* d_lh;     // adjoint: band coefficients of dL/dF, as d_uh (allocated on first use)
};

// In-kernel band forcing of the FP32 / FP16 forms.
struct FastSpectral {
    int nm;              // number of band modes (0: not used)
    int par;             // which of d_fh the next step reads
    int dirty;           // the coefficients must be recomputed from the current u
    int4* d_modes;       // kx, ky, kz, weight
    int* d_kxoff;        // first mode of each kx
    float2* d_tw[3];     // e^{i 2 pi m / n} for x, y, z
    float2* d_fh[2];     // [3][nm] synthesis coefficients
    double* d_acc;       // [16][3][nm][2] projection accumulators (copies cut atomic contention)
};

}  // namespace dl

// z planes one block of the fused kernel marches by default: the autotuner's
// choice for the 128^3 two-phase workloads in the FP32 and FP16 forms
constexpr int DL_DEFAULT_LZ = 32;

struct dl_handle {
    dl_params P;
    int nx, ny, nz;
    size_t N;
    int form;
    int device;
    cudaStream_t stream;
    int cur;                 // index of the current population / field buffer
    int64_t step;
    int force_mode;
    bool fields_set;
    bool eq_init;
    bool single;             // single-phase step (g only, DL_SINGLE_PHASE)
    char err[512];

    dl::LatticeConsts lc;
    dl::DevState* d_state;   // device scratch

    // FP64 form
    double* f64[2];          // SoA populations [15][N], two buffers
    double* g64[2];
    double* mac64[2];        // [5][N]: phi, u1, u2, u3, p
    double* rec64;           // derived records, [NREC][N]
    int nrec;
    double* force64;         // [3][N]

    // reduced precision forms (FP32 / FP16 storage)
    void* fs[2];             // populations, storage type of the form
    void* gs[2];
    float* mac32[2];         // [5][N]: phi - phi1, u1, u2, u3, p - 1/3
    float* force32;          // [3][N]
    int lz;                  // z planes per block of the fused kernel (0: DL_DEFAULT_LZ, at most nz)
    int l2_prefetch;         // fused kernel: bulk L2 prefetch of the next plane's pulls
    int sp_pipeline;         // single-phase kernel: next plane's pulls held in registers
    int proj_in_step;        // band forcing: projection of the new u inside the fused step (else its own launch)
    int push;                // FP32: step in the push form where eligible (option "push")
    int pushed;              // the state is a push step's: fields stale, band force and wall reflection pending
    int push_bulk;           // push form: next plane staged in shared memory (option "stage": 0 registers,
                             // 1 per-thread asynchronous copies, 2 tensor copies, full tiles only)
    unsigned char push_tmap[4][128];  // stage 2: tensor maps of fs[0], fs[1], gs[0], gs[1]
    int push_tmap_ok;
    long long push_wait_ns;  // stage 2: limit of a block's wait for its staged plane (option "wait_ns")
    int push_extra_tx;       // stage 2, tests of that limit: bytes expected beyond the copies' ("stage_extra_tx")
    double* mirror_dev;      // dl_set_minmax_mirror: device address of the host mirror (or null)
    long long mirror_mask;   // its slots - 1 (slots a power of two)
    // dl_energy: cuFFT plan and buffers (allocated on first use)
    long long en_plan;
    int en_plan_ok;
    double* en_buf;
    size_t en_bytes;

    dl::SpectralPlan sp;
    dl::FastSpectral fsp;
    double* d_diag;          // diagnostics partial sums
    int diag_blocks;

    // labelling scratch (labels.cu)
    int* lbl_buf;

    // adjoint (adjoint.cu)
    float* adj_lam[2];       // [30][N] adjoints of f and g
    float* adj_aux;          // [9][N]
    double* adj_grads;       // [4]
    int adj_cur;

    // launch accounting (dl_profile)
    int64_t launches;
    int prof_on;             // 0: off; n > 0: events around every n-th launch
    int prof_sample;         // the launch in flight is timed
    struct ProfEv {
        cudaEvent_t a, b;
        int main;
    } * prof;
    int prof_n, prof_cap;
};

namespace dl {
// fp64 form (step_fp64.cu)
int fp64_alloc(dl_handle* h);
void fp64_free(dl_handle* h);
int fp64_init_equilibrium(dl_handle* h);
int fp64_step(dl_handle* h);
int fp64_moments_from_populations(dl_handle* h);
// spectral forcing (spectral.cu)
int spectral_alloc(dl_handle* h);
void spectral_free(dl_handle* h);
int spectral_force_fp64(dl_handle* h, const double* d_u1, const double* d_u2, const double* d_u3,
                        double* d_fx, double* d_fy, double* d_fz);
int spectral_force_f32(dl_handle* h, const float* d_u1, const float* d_u2, const float* d_u3,
                       float* d_fx, float* d_fy, float* d_fz);
// fp32 / fp16-storage forms (step_fast.cu)
int fast_alloc(dl_handle* h);
void fast_free(dl_handle* h);
int fast_set_fields(dl_handle* h, const double* d_fields);
int fast_get_fields(dl_handle* h, double* d_fields);
int fast_init_equilibrium(dl_handle* h);
int fast_get_populations(dl_handle* h, double* d_f, double* d_g);
int fast_set_populations(dl_handle* h, const double* d_f, const double* d_g);
int fast_step(dl_handle* h);
// push form (step_push.cu)
bool push_tma_eligible(const dl_handle* h);
bool push_eligible(const dl_handle* h);
int push_step(dl_handle* h);
int fast_settle(dl_handle* h);  // complete a push step's state (no-op when settled)
// the persistent ensemble launch in the push form (step_push.cu)
size_t push_args_bytes();
void push_args_at(dl_handle* h, int k, void* out);
int launch_push_batched(dl_handle* h0, const void* table, int nm, const int4* items, int nitems,
                        const unsigned* nblk, unsigned* counter, int grid, cudaStream_t s);
int fast_prepare_force(dl_handle* h, int mode);
int spectral_project_f32(dl_handle* h, const float* d_u1, const float* d_u2, const float* d_u3);
int spectral_adjoint_f32(dl_handle* h, const float* d_lf1, const float* d_lf2, const float* d_lf3, const float* d_u1,
                         const float* d_u2, const float* d_u3, float* d_lu1, float* d_lu2, float* d_lu3);
// batched ensembles of fast-form handles (step_fast.cu)
int batch_create(dl_handle** members, int nm, void** out);
void batch_destroy(void* b);
int batch_step(void* b, int nsteps);
int batch_set_option(void* b, const char* key, long long v);
int batch_get_option(void* b, const char* key, long long* v);
// droplet labelling (labels.cu)
int label_droplets(dl_handle* h, int conn, int* labels_host, long long* ndrops, double* volumes, long long maxv);
// adjoint of the FP32 step (adjoint.cu)
int adjoint_check(dl_handle* h);
void adjoint_free(dl_handle* h);
int adjoint_begin(dl_handle* h, const float* d_lphi);
int adjoint_step(dl_handle* h, const float* d_state, long long step);
int adjoint_init(dl_handle* h, const float* d_state0, float* d_lphi0);
int adjoint_grads(dl_handle* h, double* out4);
// transposes (layout.cu)
int soa_to_aos(dl_handle* h, const double* d_soa, double* d_aos);
int aos_to_soa(dl_handle* h, const double* d_aos, double* d_soa);
int fill_doubles(dl_handle* h, double* d, double v, size_t n);
int energy_diagnostics(dl_handle* h, dl_energy_diag* out, double* spectrum_host, long long nbins);
void energy_free(dl_handle* h);
int pull_ceiling(dl_handle* h, int repeats, double* gbps);
int fp64_ceiling(dl_handle* h, double* tflops);
// diagnostics (reduce.cu)
int reduce_fields(dl_handle* h, const double* d_mac, dl_diag* out);
int reduce_fields_f32(dl_handle* h, const float* d_mac, dl_diag* out);

int set_error(dl_handle* h, int code, const char* fmt, ...);
// bracket one kernel launch: counts it and, when profiling, records events
void launch_begin(dl_handle* h);
void launch_end(dl_handle* h, bool main_kernel);
int check_cuda(dl_handle* h, cudaError_t e, const char* what);
}  // namespace dl

#define DL_LAUNCH(h, is_main, ...)        \
    do {                                  \
        dl::launch_begin(h);              \
        __VA_ARGS__;                      \
        dl::launch_end((h), (is_main));   \
    } while (0)

#define DL_CUDA(h, call)                                                  \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) return dl::check_cuda((h), e_, #call);     \
    } while (0)
