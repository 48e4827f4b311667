// dl_api.cu -- the extern "C" entry points of include/droplet_gb300.h.
// Host-side handle management, argument checking, host<->device layout
// conversion and dispatch to the form-specific kernels.
#include "dl_internal.cuh"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <new>

namespace dl {

int set_error(dl_handle* h, int code, const char* fmt, ...) {
    if (h) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(h->err, sizeof(h->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

int check_cuda(dl_handle* h, cudaError_t e, const char* what) {
    return set_error(h, DL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void launch_begin(dl_handle* h) {
    h->prof_sample = h->prof_on && (h->launches % h->prof_on) == 0;
    if (!h->prof_sample) return;
    if (h->prof_n == h->prof_cap) {
        int cap = h->prof_cap ? 2 * h->prof_cap : 256;
        void* p = realloc(h->prof, sizeof(dl_handle::ProfEv) * cap);
        if (!p) {
            h->prof_on = 0;
            h->prof_sample = 0;
            return;
        }
        h->prof = (dl_handle::ProfEv*)p;
        for (int k = h->prof_cap; k < cap; ++k) {
            cudaEventCreate(&h->prof[k].a);
            cudaEventCreate(&h->prof[k].b);
        }
        h->prof_cap = cap;
    }
    cudaEventRecord(h->prof[h->prof_n].a, h->stream);
}

void launch_end(dl_handle* h, bool main_kernel) {
    h->launches += 1;
    if (!h->prof_sample) return;
    h->prof_sample = 0;
    cudaEventRecord(h->prof[h->prof_n].b, h->stream);
    h->prof[h->prof_n].main = main_kernel ? 1 : 0;
    h->prof_n += 1;
}

static void prof_release(dl_handle* h) {
    for (int k = 0; k < h->prof_cap; ++k) {
        cudaEventDestroy(h->prof[k].a);
        cudaEventDestroy(h->prof[k].b);
    }
    free(h->prof);
    h->prof = nullptr;
    h->prof_cap = h->prof_n = 0;
}

static void init_consts(dl_handle* h) {
    // program/lbm_drop_xy.f90:77-84, each entry rounded as the reference rounds it
    const double E[Q] = {2.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,
                         1.0 / 9.0,  1.0 / 9.0,  1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0,
                         1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0};
    const double F[Q] = {-7.0 / 3.0, 1.0 / 3.0,  1.0 / 3.0,  1.0 / 3.0,  1.0 / 3.0,
                         1.0 / 3.0,  1.0 / 3.0,  1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0,
                         1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0};
    for (int i = 0; i < Q; ++i) {
        h->lc.E[i] = E[i];
        h->lc.F[i] = F[i];
        h->lc.Ekf[i] = E[i] * h->P.kappaf;
        h->lc.Ekg[i] = E[i] * h->P.kappag;
        h->lc.ds3E[i] = (3.0 * h->P.ds) * E[i];
        h->lc.six_E[i] = 6.0 * E[i];
    }
}

static int reset_state(dl_handle* h) {
    DevState s;
    memset(&s, 0, sizeof(s));
    s.phi_min = h->P.phi1;
    s.phi_max = h->P.phi2;
    s.key_min = KEY_POS_INF;
    s.key_max = KEY_NEG_INF;
    DL_CUDA(h, cudaMemcpyAsync(h->d_state, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    return DL_OK;
}

static int set_minmax(dl_handle* h, double mn, double mx) {
    double v[2] = {mn, mx};
    DL_CUDA(h, cudaMemcpyAsync(h->d_state, v, sizeof(v), cudaMemcpyHostToDevice, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    return DL_OK;
}

// Device scratch for a host<->device transfer of one SoA array set.
struct Staging {
    double* d = nullptr;
    ~Staging() {
        if (d) cudaFree(d);
    }
};

static bool is_fast(const dl_handle* h) { return h->form == DL_FORM_FP32 || h->form == DL_FORM_FP16; }

// a push step leaves phi, u, p stale and the band force and wall reflection of
// its streaming pending: everything that reads the state settles it first
static int settled(dl_handle* h) { return (is_fast(h) && h->pushed) ? fast_settle(h) : DL_OK; }

__global__ void f64_to_f32(const double* __restrict__ a, float* __restrict__ b, long long n) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) b[t] = (float)a[t];
}

}  // namespace dl

using namespace dl;

extern "C" {

int dl_version(void) { return 100; }

const char* dl_status_string(int status) {
    switch (status) {
        case DL_OK: return "ok";
        case DL_ERR_ARG: return "bad argument";
        case DL_ERR_CUDA: return "CUDA error";
        case DL_ERR_ALLOC: return "allocation failed";
        case DL_ERR_NAN: return "NaN/Inf detected";
        case DL_ERR_TIMEOUT: return "device wait timed out";
        case DL_ERR_STATE: return "call out of order";
        case DL_ERR_UNSUPPORTED: return "unsupported option for this form";
        default: return "unknown status";
    }
}

int dl_create(const dl_params* params, int nx, int ny, int nz, int form, dl_handle** out) {
    if (!params || !out) return DL_ERR_ARG;
    *out = nullptr;
    if (nx < 3 || ny < 3 || nz < 3) return DL_ERR_ARG;
    const bool single = (form & DL_SINGLE_PHASE) != 0;
    form &= ~DL_SINGLE_PHASE;
    if (form != DL_FORM_FP64 && form != DL_FORM_FP32 && form != DL_FORM_FP16) return DL_ERR_UNSUPPORTED;
    if (single && (params->les != 0 || params->Anu != 0.0)) return DL_ERR_UNSUPPORTED;
    // the A_nu strain term of geq (program/lbm_drop_xy.f90:461-469) is in the FP64 form only
    if (form != DL_FORM_FP64 && params->Anu != 0.0) return DL_ERR_UNSUPPORTED;
    if (params->tauf <= 0.5 || params->ds <= 0.0 || params->phi2 == params->phi1) return DL_ERR_ARG;
    if (params->kc < 0 || params->visc_mode < 0 || params->visc_mode > 1) return DL_ERR_ARG;
    dl_handle* h = new (std::nothrow) dl_handle();
    if (!h) return DL_ERR_ALLOC;
    memset(h, 0, sizeof(*h));
    h->P = *params;
    h->nx = nx;
    h->ny = ny;
    h->nz = nz;
    h->N = (size_t)nx * ny * nz;
    h->form = form;
    h->single = single;
    // L2 prefetch of the next plane's pulled rows: pays off where arithmetic,
    // not bandwidth, sets the pace (the two-phase FP32 step); "prefetch" option
    h->l2_prefetch = (!single && form == DL_FORM_FP32) ? 1 : 0;
    // band forcing: the new u is projected by each block of the fused step
    // after its march ("projection" option; 0: a launch of its own)
    h->proj_in_step = 1;
    // FP32: the push form where eligible (push_eligible)
    h->push = (form == DL_FORM_FP32) ? 1 : 0;
    // push form: staging the next plane in shared memory pays for the single-phase
    // step (no stencils: little work to hide the loads behind), not the two-phase one
    h->push_bulk = single ? 1 : 0;
    h->push_wait_ns = 2000000000LL;
    if (single) {
        // the precursor step: constant nu1, no interface terms
        h->P.kappaf = 0.0;
        h->P.kappag = 0.0;
        h->P.nu2 = h->P.nu1;
        h->P.visc_mode = DL_VISC_FIXED;
    }
    h->stream = 0;
    h->force_mode = DL_FORCE_NONE;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) {
        delete h;
        return DL_ERR_CUDA;
    }
    init_consts(h);
    int rc = DL_OK;
    if (cudaMalloc(&h->d_state, sizeof(DevState)) != cudaSuccess) rc = DL_ERR_ALLOC;
    if (rc == DL_OK) rc = reset_state(h);
    if (rc == DL_OK) rc = is_fast(h) ? fast_alloc(h) : fp64_alloc(h);
    if (rc == DL_OK) rc = spectral_alloc(h);
    if (rc != DL_OK) {
        dl_destroy(h);
        return rc == DL_ERR_CUDA ? DL_ERR_ALLOC : rc;
    }
    *out = h;
    return DL_OK;
}

int dl_destroy(dl_handle* h) {
    if (!h) return DL_ERR_ARG;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    fp64_free(h);
    fast_free(h);
    adjoint_free(h);
    spectral_free(h);
    cudaFree(h->d_state);
    cudaFree(h->d_diag);
    cudaFree(h->lbl_buf);
    energy_free(h);
    prof_release(h);
    delete h;
    return DL_OK;
}

int dl_profile(dl_handle* h, int enable) {
    if (!h) return DL_ERR_ARG;
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    if (enable < 0) return set_error(h, DL_ERR_ARG, "dl_profile: enable must be >= 0");
    h->prof_on = enable;
    h->prof_sample = 0;
    h->prof_n = 0;
    h->launches = 0;
    return DL_OK;
}

int dl_profile_read(dl_handle* h, dl_profile_stats* out) {
    if (!h || !out) return DL_ERR_ARG;
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    memset(out, 0, sizeof(*out));
    for (int k = 0; k < h->prof_n; ++k) {
        float ms = 0.f;
        DL_CUDA(h, cudaEventElapsedTime(&ms, h->prof[k].a, h->prof[k].b));
        out->total_ms += ms;
        out->timed_launches += 1;
        if (h->prof[k].main) {
            out->main_ms += ms;
            out->main_launches += 1;
        }
    }
    out->launches = h->launches;
    h->prof_n = 0;
    h->launches = 0;
    return DL_OK;
}

int dl_label_droplets(dl_handle* h, int connectivity, int32_t* labels, int64_t* ndrops, double* volumes,
                      int64_t max_volumes) {
    if (!h || !ndrops || (max_volumes > 0 && !volumes) || max_volumes < 0) return DL_ERR_ARG;
    if (h->single) return set_error(h, DL_ERR_UNSUPPORTED, "no droplets in the single-phase step");
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    long long n = 0;
    int rc = label_droplets(h, connectivity, (int*)labels, &n, volumes, (long long)max_volumes);
    *ndrops = (int64_t)n;
    return rc;
}

int dl_state_floats(dl_handle* h, int64_t* n) {
    if (!h || !n) return DL_ERR_ARG;
    if (h->form != DL_FORM_FP32 || h->single)
        return set_error(h, DL_ERR_UNSUPPORTED, "device state export is for the two-phase FP32 form");
    *n = (int64_t)35 * (int64_t)h->N;
    return DL_OK;
}

int dl_save_state(dl_handle* h, void* d_dst) {
    if (!h || !d_dst) return DL_ERR_ARG;
    if (h->form != DL_FORM_FP32 || h->single)
        return set_error(h, DL_ERR_UNSUPPORTED, "device state export is for the two-phase FP32 form");
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    const size_t N = h->N;
    float* d = (float*)d_dst;
    DL_CUDA(h, cudaMemcpyAsync(d, h->fs[h->cur], sizeof(float) * Q * N, cudaMemcpyDeviceToDevice, h->stream));
    DL_CUDA(h, cudaMemcpyAsync(d + Q * N, h->gs[h->cur], sizeof(float) * Q * N, cudaMemcpyDeviceToDevice, h->stream));
    DL_CUDA(h, cudaMemcpyAsync(d + 2 * Q * N, h->mac32[h->cur], sizeof(float) * 5 * N, cudaMemcpyDeviceToDevice,
                               h->stream));
    return DL_OK;
}

int dl_load_state(dl_handle* h, const void* d_src) {
    if (!h || !d_src) return DL_ERR_ARG;
    if (h->form != DL_FORM_FP32 || h->single)
        return set_error(h, DL_ERR_UNSUPPORTED, "device state import is for the two-phase FP32 form");
    const size_t N = h->N;
    const float* d = (const float*)d_src;
    DL_CUDA(h, cudaMemcpyAsync(h->fs[h->cur], d, sizeof(float) * Q * N, cudaMemcpyDeviceToDevice, h->stream));
    DL_CUDA(h, cudaMemcpyAsync(h->gs[h->cur], d + Q * N, sizeof(float) * Q * N, cudaMemcpyDeviceToDevice, h->stream));
    DL_CUDA(h, cudaMemcpyAsync(h->mac32[h->cur], d + 2 * Q * N, sizeof(float) * 5 * N, cudaMemcpyDeviceToDevice,
                               h->stream));
    h->fields_set = true;
    h->eq_init = true;
    h->pushed = 0;
    // the band coefficients of the next step come from the loaded u
    if (h->force_mode == DL_FORCE_SPECTRAL) h->fsp.dirty = 1;
    return DL_OK;
}

int dl_adjoint_state_floats(dl_handle* h, int64_t* n) {
    if (!h || !n) return DL_ERR_ARG;
    if (h->form != DL_FORM_FP32 || h->single)
        return set_error(h, DL_ERR_UNSUPPORTED, "device state export is for the two-phase FP32 form");
    // f, fields (, g: the adjoint of a per-site tau_g, LES or a viscosity ratio, reads it)
    *n = (int64_t)((h->P.les || h->P.nu2 != h->P.nu1) ? 35 : 20) * (int64_t)h->N;
    return DL_OK;
}

int dl_save_adjoint_state(dl_handle* h, void* d_dst) {
    if (!h || !d_dst) return DL_ERR_ARG;
    if (h->form != DL_FORM_FP32 || h->single)
        return set_error(h, DL_ERR_UNSUPPORTED, "device state export is for the two-phase FP32 form");
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    const size_t N = h->N;
    float* d = (float*)d_dst;
    DL_CUDA(h, cudaMemcpyAsync(d, h->fs[h->cur], sizeof(float) * Q * N, cudaMemcpyDeviceToDevice, h->stream));
    DL_CUDA(h, cudaMemcpyAsync(d + Q * N, h->mac32[h->cur], sizeof(float) * 5 * N, cudaMemcpyDeviceToDevice,
                               h->stream));
    if (h->P.les || h->P.nu2 != h->P.nu1)
        DL_CUDA(h, cudaMemcpyAsync(d + 20 * N, h->gs[h->cur], sizeof(float) * Q * N, cudaMemcpyDeviceToDevice,
                                   h->stream));
    return DL_OK;
}

int dl_adjoint_begin(dl_handle* h, const float* d_dloss_dphi) {
    if (!h || !d_dloss_dphi) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    return adjoint_begin(h, d_dloss_dphi);
}

int dl_adjoint_step(dl_handle* h, const void* d_state_before, int64_t step) {
    if (!h || !d_state_before || step < 1) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    return adjoint_step(h, (const float*)d_state_before, (long long)step);
}

int dl_adjoint_init(dl_handle* h, const void* d_state0, float* d_dloss_dphi0) {
    if (!h || !d_state0 || !d_dloss_dphi0) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    return adjoint_init(h, (const float*)d_state0, d_dloss_dphi0);
}

int dl_adjoint_grads(dl_handle* h, double* grads) {
    if (!h || !grads) return DL_ERR_ARG;
    return adjoint_grads(h, grads);
}

int dl_set_option(dl_handle* h, const char* key, int64_t value) {
    if (!h || !key) return DL_ERR_ARG;
    if (strcmp(key, "lz") == 0) {
        if (value < 0 || value > h->nz) return set_error(h, DL_ERR_ARG, "lz=%lld outside 0..nz", (long long)value);
        h->lz = value == 0 ? (h->nz < DL_DEFAULT_LZ ? h->nz : DL_DEFAULT_LZ) : (int)value;
        return DL_OK;
    }
    if (strcmp(key, "prefetch") == 0) {
        if (value < 0 || value > 1) return set_error(h, DL_ERR_ARG, "prefetch must be 0 or 1");
        h->l2_prefetch = (int)value;
        return DL_OK;
    }
    if (strcmp(key, "pipeline") == 0) {
        if (value < 0 || value > 1) return set_error(h, DL_ERR_ARG, "pipeline must be 0 or 1");
        h->sp_pipeline = (int)value;
        return DL_OK;
    }
    if (strcmp(key, "projection") == 0) {
        if (value < 0 || value > 1) return set_error(h, DL_ERR_ARG, "projection must be 0 or 1");
        h->proj_in_step = (int)value;
        return DL_OK;
    }
    if (strcmp(key, "push") == 0) {
        if (value < 0 || value > 1) return set_error(h, DL_ERR_ARG, "push must be 0 or 1");
        h->push = (int)value;
        return DL_OK;
    }
    if (strcmp(key, "stage") == 0) {
        if (value < 0 || value > 2) return set_error(h, DL_ERR_ARG, "stage must be 0, 1 or 2");
        if (value == 2 && !push_tma_eligible(h))
            return set_error(h, DL_ERR_UNSUPPORTED, "stage 2 (tensor copies) needs nx a multiple of 32 and ny of 8");
        h->push_bulk = (int)value;
        return DL_OK;
    }
    if (strcmp(key, "wait_ns") == 0) {
        if (value < 1000 || value > 60000000000LL) return set_error(h, DL_ERR_ARG, "wait_ns must be in [1e3, 6e10]");
        h->push_wait_ns = value;
        return DL_OK;
    }
    if (strcmp(key, "stage_extra_tx") == 0) {
        if (value < 0 || value > 4096 || value % 16) return set_error(h, DL_ERR_ARG, "stage_extra_tx must be 0 .. 4096, a multiple of 16");
        h->push_extra_tx = (int)value;
        return DL_OK;
    }
    return set_error(h, DL_ERR_ARG, "unknown option '%s'", key);
}

int dl_get_option(dl_handle* h, const char* key, int64_t* value) {
    if (!h || !key || !value) return DL_ERR_ARG;
    if (strcmp(key, "lz") == 0) {
        *value = h->lz;
        return DL_OK;
    }
    if (strcmp(key, "prefetch") == 0) {
        *value = h->l2_prefetch;
        return DL_OK;
    }
    if (strcmp(key, "pipeline") == 0) {
        *value = h->sp_pipeline;
        return DL_OK;
    }
    if (strcmp(key, "projection") == 0) {
        *value = h->proj_in_step;
        return DL_OK;
    }
    if (strcmp(key, "push") == 0) {
        *value = h->push;
        return DL_OK;
    }
    if (strcmp(key, "stage") == 0) {
        *value = h->push_bulk;
        return DL_OK;
    }
    if (strcmp(key, "wait_ns") == 0) {
        *value = h->push_wait_ns;
        return DL_OK;
    }
    if (strcmp(key, "stage_extra_tx") == 0) {
        *value = h->push_extra_tx;
        return DL_OK;
    }
    if (strcmp(key, "push_eligible") == 0) {  // read only: the next step takes the push form
        *value = (h->form == DL_FORM_FP32 && push_eligible(h)) ? 1 : 0;
        return DL_OK;
    }
    if (strcmp(key, "pushed") == 0) {  // read only: the state awaits its settle
        *value = h->pushed;
        return DL_OK;
    }
    return set_error(h, DL_ERR_ARG, "unknown option '%s'", key);
}

int dl_set_stream(dl_handle* h, void* stream) {
    if (!h) return DL_ERR_ARG;
    h->stream = (cudaStream_t)stream;
    return DL_OK;
}

int dl_set_fields(dl_handle* h, const double* phi, const double* u1, const double* u2, const double* u3,
                  const double* p) {
    if (!h || !phi || !u1 || !u2 || !u3 || !p) return DL_ERR_ARG;
    const size_t N = h->N;
    Staging st;
    double* d = h->mac64[h->cur];
    if (is_fast(h)) {
        DL_CUDA(h, cudaMalloc(&st.d, 5 * N * sizeof(double)));
        d = st.d;
    }
    const double* src[5] = {phi, u1, u2, u3, p};
    for (int k = 0; k < 5; ++k) {
        if (k == 0 && h->single) {  // single phase: phi is not a field
            int rc = fill_doubles(h, d, h->P.phi1, N);
            if (rc != DL_OK) return rc;
            continue;
        }
        DL_CUDA(h, cudaMemcpyAsync(d + k * N, src[k], N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    }
    if (is_fast(h)) {
        int rc = fast_set_fields(h, d);
        if (rc != DL_OK) return rc;
    }
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    h->fields_set = true;
    h->pushed = 0;
    return DL_OK;
}

int dl_get_fields(dl_handle* h, double* phi, double* u1, double* u2, double* u3, double* p) {
    if (!h || !phi || !u1 || !u2 || !u3 || !p) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    const size_t N = h->N;
    Staging st;
    const double* d = h->mac64[h->cur];
    if (is_fast(h)) {
        DL_CUDA(h, cudaMalloc(&st.d, 5 * N * sizeof(double)));
        int rc = fast_get_fields(h, st.d);
        if (rc != DL_OK) return rc;
        d = st.d;
    }
    double* dst[5] = {phi, u1, u2, u3, p};
    for (int k = 0; k < 5; ++k)
        DL_CUDA(h, cudaMemcpyAsync(dst[k], d + k * N, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    return DL_OK;
}

int dl_init_equilibrium(dl_handle* h) {
    if (!h) return DL_ERR_ARG;
    if (!h->fields_set) return set_error(h, DL_ERR_STATE, "dl_init_equilibrium before dl_set_fields");
    int rc = set_minmax(h, h->P.phi1, h->P.phi2);
    if (rc != DL_OK) return rc;
    rc = is_fast(h) ? fast_init_equilibrium(h) : fp64_init_equilibrium(h);
    if (rc != DL_OK) return rc;
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    h->eq_init = true;
    h->pushed = 0;
    return DL_OK;
}

int dl_set_force(dl_handle* h, int mode, const double* fx, const double* fy, const double* fz) {
    if (!h) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    const size_t N = h->N;
    if (mode != DL_FORCE_NONE && mode != DL_FORCE_STATIC && mode != DL_FORCE_SPECTRAL) return DL_ERR_ARG;
    if (mode == DL_FORCE_SPECTRAL && (h->P.kc < 2 || h->sp.K < 1))
        return set_error(h, DL_ERR_ARG,
                         "spectral forcing needs kc >= 2 and a domain holding the band (2 kc - 1 <= nx, ny; "
                         "kc <= nz / 2)");
    if (is_fast(h) && mode != DL_FORCE_NONE && h->P.ds != 1.0)
        return set_error(h, DL_ERR_UNSUPPORTED, "the FP32 and FP16 forms apply a body force at ds = 1 only");
    if (is_fast(h)) {
        int rc = fast_prepare_force(h, mode);
        if (rc != DL_OK) return rc;
    }
    if (mode == DL_FORCE_STATIC) {
        if (!fx || !fy || !fz) return DL_ERR_ARG;
        const double* src[3] = {fx, fy, fz};
        if (is_fast(h)) {
            Staging st;
            DL_CUDA(h, cudaMalloc(&st.d, 3 * N * sizeof(double)));
            for (int k = 0; k < 3; ++k)
                DL_CUDA(h, cudaMemcpyAsync(st.d + k * N, src[k], N * sizeof(double), cudaMemcpyHostToDevice,
                                           h->stream));
            f64_to_f32<<<(unsigned)((3 * N + 255) / 256), 256, 0, h->stream>>>(st.d, h->force32, (long long)(3 * N));
            DL_CUDA(h, cudaGetLastError());
            DL_CUDA(h, cudaStreamSynchronize(h->stream));
        } else {
            for (int k = 0; k < 3; ++k)
                DL_CUDA(h, cudaMemcpyAsync(h->force64 + k * N, src[k], N * sizeof(double), cudaMemcpyHostToDevice,
                                           h->stream));
        }
    } else if (mode == DL_FORCE_NONE || mode == DL_FORCE_SPECTRAL) {
        if (is_fast(h)) {
            if (h->force32) DL_CUDA(h, cudaMemsetAsync(h->force32, 0, 3 * N * sizeof(float), h->stream));
        }
        else DL_CUDA(h, cudaMemsetAsync(h->force64, 0, 3 * N * sizeof(double), h->stream));
    } else {
        return DL_ERR_ARG;
    }
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    h->force_mode = mode;
    return DL_OK;
}

// one warp after a step: its phi range into slot `slot` of the host mirror. A
// launch of its own, because any code added to the step kernels' shared
// finalisation changes their register allocation (a store there made the FP16
// step 5 % slower)
__global__ void mirror_copy(const DevState* __restrict__ st, double* __restrict__ m, long long slot) {
    if (threadIdx.x == 0) {
        m[2 * slot] = st->phi_min;
        m[2 * slot + 1] = st->phi_max;
    }
}

int dl_step(dl_handle* h, int nsteps) {
    if (!h || nsteps < 0) return DL_ERR_ARG;
    if (!h->eq_init) return set_error(h, DL_ERR_STATE, "dl_step before dl_init_equilibrium / dl_set_populations");
    for (int k = 0; k < nsteps; ++k) {
        int rc = is_fast(h) ? fast_step(h) : fp64_step(h);
        if (rc != DL_OK) return rc;
        if (h->mirror_dev) {
            // a push step reduces the range of the state it loaded, the previous step's
            const long long at = h->pushed ? h->step - 1 : h->step;
            DL_LAUNCH(h, false, (mirror_copy<<<1, 32, 0, h->stream>>>(h->d_state, h->mirror_dev, at & h->mirror_mask)));
            DL_CUDA(h, cudaGetLastError());
        }
    }
    return DL_OK;
}

int dl_get_populations(dl_handle* h, double* f, double* g) {
    if (!h || !f || !g) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    const size_t bytes = Q * h->N * sizeof(double);
    Staging st;
    if (is_fast(h)) {
        DL_CUDA(h, cudaMalloc(&st.d, 2 * bytes));
        int rc = fast_get_populations(h, st.d, st.d + Q * h->N);
        if (rc != DL_OK) return rc;
        DL_CUDA(h, cudaMemcpyAsync(f, st.d, bytes, cudaMemcpyDeviceToHost, h->stream));
        DL_CUDA(h, cudaMemcpyAsync(g, st.d + Q * h->N, bytes, cudaMemcpyDeviceToHost, h->stream));
        DL_CUDA(h, cudaStreamSynchronize(h->stream));
        return DL_OK;
    }
    DL_CUDA(h, cudaMalloc(&st.d, bytes));
    int rc = DL_OK;
    if (h->single) {
        memset(f, 0, bytes);  // single phase: no f
    } else {
        rc = soa_to_aos(h, h->f64[h->cur], st.d);
        if (rc != DL_OK) return rc;
        DL_CUDA(h, cudaMemcpyAsync(f, st.d, bytes, cudaMemcpyDeviceToHost, h->stream));
        DL_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    rc = soa_to_aos(h, h->g64[h->cur], st.d);
    if (rc != DL_OK) return rc;
    DL_CUDA(h, cudaMemcpyAsync(g, st.d, bytes, cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    return DL_OK;
}

int dl_set_populations(dl_handle* h, const double* f, const double* g) {
    if (!h || !f || !g) return DL_ERR_ARG;
    const size_t bytes = Q * h->N * sizeof(double);
    Staging st;
    if (is_fast(h)) {
        DL_CUDA(h, cudaMalloc(&st.d, 2 * bytes));
        DL_CUDA(h, cudaMemcpyAsync(st.d, f, bytes, cudaMemcpyHostToDevice, h->stream));
        DL_CUDA(h, cudaMemcpyAsync(st.d + Q * h->N, g, bytes, cudaMemcpyHostToDevice, h->stream));
        int rc = fast_set_populations(h, st.d, st.d + Q * h->N);
        if (rc != DL_OK) return rc;
        DL_CUDA(h, cudaStreamSynchronize(h->stream));
        h->fields_set = true;
        h->eq_init = true;
        return DL_OK;
    }
    DL_CUDA(h, cudaMalloc(&st.d, bytes));
    int rc = DL_OK;
    if (!h->single) {  // single phase: f is ignored
        DL_CUDA(h, cudaMemcpyAsync(st.d, f, bytes, cudaMemcpyHostToDevice, h->stream));
        rc = aos_to_soa(h, st.d, h->f64[h->cur]);
        if (rc != DL_OK) return rc;
        DL_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    DL_CUDA(h, cudaMemcpyAsync(st.d, g, bytes, cudaMemcpyHostToDevice, h->stream));
    rc = aos_to_soa(h, st.d, h->g64[h->cur]);
    if (rc != DL_OK) return rc;
    rc = fp64_moments_from_populations(h);
    if (rc != DL_OK) return rc;
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    h->fields_set = true;
    h->eq_init = true;
    return DL_OK;
}

int dl_set_step(dl_handle* h, int64_t step) {
    if (!h || step < 0) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    h->step = step;
    return DL_OK;
}

int dl_get_step(dl_handle* h, int64_t* step) {
    if (!h || !step) return DL_ERR_ARG;
    *step = h->step;
    return DL_OK;
}

int dl_get_minmax(dl_handle* h, double* mn, double* mx) {
    if (!h || !mn || !mx) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    double v[2];
    DL_CUDA(h, cudaMemcpyAsync(v, h->d_state, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    *mn = v[0];
    *mx = v[1];
    return DL_OK;
}

int dl_get_minmax_async(dl_handle* h, double* dst) {
    if (!h || !dst) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    // phi_min and phi_max are the first two fields of the device state
    DL_CUDA(h, cudaMemcpyAsync(dst, h->d_state, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return DL_OK;
}

int dl_set_minmax_mirror(dl_handle* h, double* host, int64_t nslots) {
    if (!h) return DL_ERR_ARG;
    double* dev = nullptr;
    if (host) {
        if (nslots < 1 || (nslots & (nslots - 1)))
            return set_error(h, DL_ERR_ARG, "minmax mirror: nslots must be a power of two");
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, host) != cudaSuccess || at.type != cudaMemoryTypeHost ||
            !at.devicePointer) {
            cudaGetLastError();
            return set_error(h, DL_ERR_ARG, "minmax mirror: not page-locked host memory the device can write");
        }
        dev = (double*)at.devicePointer;
    }
    h->mirror_dev = dev;
    h->mirror_mask = dev ? nslots - 1 : 0;
    return DL_OK;
}

int dl_host_alloc(int64_t bytes, void** out) {
    if (!out || bytes < 0) return DL_ERR_ARG;
    *out = nullptr;
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes > 0 ? (size_t)bytes : 1, cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        return DL_ERR_ALLOC;
    }
    memset(p, 0, bytes > 0 ? (size_t)bytes : 1);
    *out = p;
    return DL_OK;
}

int dl_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) {
        cudaGetLastError();
        return DL_ERR_ARG;
    }
    return DL_OK;
}

int dl_sync(dl_handle* h) {
    if (!h) return DL_ERR_ARG;
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    DevState s;
    DL_CUDA(h, cudaMemcpy(&s, h->d_state, sizeof(s), cudaMemcpyDeviceToHost));
    if (s.wait_timeout) return set_error(h, DL_ERR_TIMEOUT, "a tensor copy of the staged plane did not complete in time");
    if (s.nan_flag) return set_error(h, DL_ERR_NAN, "non-finite phi/u/p first seen at step %lld", s.nan_step);
    return DL_OK;
}

int dl_energy(dl_handle* h, dl_energy_diag* out, double* spectrum, int64_t nbins) {
    if (!h || !out) return DL_ERR_ARG;
    if (!h->fields_set) return set_error(h, DL_ERR_STATE, "dl_energy before dl_set_fields");
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    return energy_diagnostics(h, out, spectrum, (long long)nbins);
}

int dl_pull_ceiling(dl_handle* h, int repeats, double* gbps) {
    if (!h || !gbps) return DL_ERR_ARG;
    return pull_ceiling(h, repeats, gbps);
}

int dl_fp64_ceiling(dl_handle* h, double* tflops) {
    if (!h || !tflops) return DL_ERR_ARG;
    return fp64_ceiling(h, tflops);
}

int dl_reduce(dl_handle* h, dl_diag* out) {
    if (!h || !out) return DL_ERR_ARG;
    {
        const int src = settled(h);
        if (src != DL_OK) return src;
    }
    int rc = is_fast(h) ? reduce_fields_f32(h, h->mac32[h->cur], out) : reduce_fields(h, h->mac64[h->cur], out);
    if (rc != DL_OK) return rc;
    DevState s;
    DL_CUDA(h, cudaMemcpy(&s, h->d_state, sizeof(s), cudaMemcpyDeviceToHost));
    out->step = h->step;
    out->nan_flag = s.nan_flag;
    return DL_OK;
}

int dl_last_error(dl_handle* h, char* buf, int buflen) {
    if (!h || !buf || buflen <= 0) return DL_ERR_ARG;
    snprintf(buf, (size_t)buflen, "%s", h->err);
    return DL_OK;
}

}  // extern "C"

// ---- batched ensembles ------------------------------------------------------
struct dl_batch {
    int nm;
    dl_handle** mem;
    void* impl;
};

extern "C" {

int dl_batch_create(const dl_params* params, const int* dims, int nmembers, int form, dl_batch** out) {
    if (!params || !dims || !out || nmembers < 1) return DL_ERR_ARG;
    *out = nullptr;
    if (form != DL_FORM_FP32 && form != DL_FORM_FP16) return DL_ERR_UNSUPPORTED;
    for (int m = 1; m < nmembers; ++m)
        if ((params[m].les != 0) != (params[0].les != 0)) return DL_ERR_ARG;
    dl_batch* b = new (std::nothrow) dl_batch();
    if (!b) return DL_ERR_ALLOC;
    b->nm = nmembers;
    b->mem = (dl_handle**)calloc((size_t)nmembers, sizeof(dl_handle*));
    if (!b->mem) {
        delete b;
        return DL_ERR_ALLOC;
    }
    int rc = DL_OK;
    for (int m = 0; m < nmembers && rc == DL_OK; ++m)
        rc = dl_create(&params[m], dims[3 * m], dims[3 * m + 1], dims[3 * m + 2], form, &b->mem[m]);
    if (rc == DL_OK) rc = batch_create(b->mem, nmembers, &b->impl);
    if (rc != DL_OK) {
        dl_batch_destroy(b);
        return rc;
    }
    *out = b;
    return DL_OK;
}

int dl_batch_member(dl_batch* b, int m, dl_handle** member) {
    if (!b || !member || m < 0 || m >= b->nm) return DL_ERR_ARG;
    *member = b->mem[m];
    return DL_OK;
}

int dl_batch_set_stream(dl_batch* b, void* stream) {
    if (!b) return DL_ERR_ARG;
    for (int m = 0; m < b->nm; ++m) b->mem[m]->stream = (cudaStream_t)stream;
    return DL_OK;
}

int dl_batch_step(dl_batch* b, int nsteps) {
    if (!b || nsteps < 0) return DL_ERR_ARG;
    return batch_step(b->impl, nsteps);
}

int dl_batch_set_option(dl_batch* b, const char* key, int64_t value) {
    if (!b || !key) return DL_ERR_ARG;
    return batch_set_option(b->impl, key, (long long)value);
}

int dl_batch_get_option(dl_batch* b, const char* key, int64_t* value) {
    if (!b || !key || !value) return DL_ERR_ARG;
    long long v = 0;
    int rc = batch_get_option(b->impl, key, &v);
    if (rc == DL_OK) *value = (int64_t)v;
    return rc;
}

int dl_batch_destroy(dl_batch* b) {
    if (!b) return DL_ERR_ARG;
    if (b->impl) batch_destroy(b->impl);
    for (int m = 0; m < b->nm; ++m)
        if (b->mem[m]) dl_destroy(b->mem[m]);
    free(b->mem);
    delete b;
    return DL_OK;
}

}  // extern "C"
