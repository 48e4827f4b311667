// reduce_static.cu -- dl_reduce_static: the whole-domain diagnostics of
// dl_reduce (same sums, same formulas) in a single launch whose working
// memory is one fixed array compiled into this library. The call allocates
// no device memory: no cudaMalloc, no cudaFree, no allocating library
// routine, and it skips the launch-event profiling (whose event pool may
// grow). It serves callers that must not allocate once a run is set up,
// for instance a host program that reserves nearly all of the GPU's memory
// for its lattices up front and would fail (or have to give memory back) on
// the few-kilobyte buffer that dl_reduce takes on its first call, or a
// monitoring thread that must not enter the device allocator while other
// threads keep stepping.
//
// The array is shared by every handle on a device. Calls that overlap in
// time on one device (from two streams, two handles or two host threads)
// race on it and give wrong sums: the caller serialises them.
//
// The array's device address belongs to the CUDA context that loaded this
// library's module. It is looked up on the first call in each context of a
// device and kept with that context's id; after a cudaDeviceReset (a new
// primary context, the module loaded again, possibly elsewhere) the next call
// looks it up again.
#include "dl_internal.cuh"
#include "diag_site.cuh"

#include <cuda.h>
#include <mutex>
#include <string.h>

namespace dl {

constexpr int RS_NSUM = DIAG_NSUM;  // sums, then min, max (the dl_reduce set)
constexpr int RS_NPART = RS_NSUM + 2;
constexpr int RS_THREADS = 256;
constexpr int RS_MAX_BLOCKS = DL_REDUCE_STATIC_MAX_BLOCKS;
constexpr int RS_DEFAULT_BLOCKS = 304;  // 2 x 152 SMs
constexpr int RS_SEGS = 8;              // block-order segments of the final sum
static_assert(RS_NPART * RS_SEGS <= RS_THREADS, "the last block folds one (value, segment) pair per thread");

// Layout, in doubles: [0, RS_MAX_BLOCKS * RS_NPART) per-block partials,
// then RS_NPART results, then one 64-bit arrival counter. 253,144 bytes.
// Nothing in the partials or the results has to start at zero: every call
// writes them before it reads them. The counter must be zero when the
// launch starts: every call clears it on its stream just before the launch
// (an 8-byte memset, which allocates nothing), and the last block of a
// launch that ran to its end also puts it back to zero.
constexpr size_t RS_WORDS = (size_t)RS_MAX_BLOCKS * RS_NPART + RS_NPART + 1;
static __device__ __align__(256) double g_reduce_scratch[RS_WORDS];

static_assert(RS_WORDS * sizeof(double) == DL_REDUCE_STATIC_SCRATCH_BYTES, "scratch size and header disagree");

struct RsArgs {
    DiagConsts k;
};

// Neumaier step: (s, c) += v
__device__ __forceinline__ void rs_add(double& s, double& c, double v) {
    const double t = s + v;
    if (fabs(s) >= fabs(v)) c += (s - t) + v;
    else c += (v - t) + s;
    s = t;
}

template <typename T>
__global__ void __launch_bounds__(RS_THREADS) reduce_static_kernel(const T* __restrict__ mac, const RsArgs a,
                                                                   double* __restrict__ scratch) {
    double* part = scratch;
    double* result = scratch + (size_t)RS_MAX_BLOCKS * RS_NPART;
    unsigned long long* arrivals = reinterpret_cast<unsigned long long*>(result + RS_NPART);

    double acc[RS_NSUM];
#pragma unroll
    for (int k = 0; k < RS_NSUM; ++k) acc[k] = 0.0;
    double vmin = INFINITY, vmax = -INFINITY;
    diag_sites(mac, a.k, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, acc, vmin,
               vmax);

    // block partials: warp shuffles, then one row per warp in shared memory
    __shared__ double sh[RS_THREADS / 32][RS_NPART];
    __shared__ double seg_s[RS_NPART][RS_SEGS], seg_c[RS_NPART][RS_SEGS];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < RS_NSUM; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][k] = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vmin = fmin(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    if (lane == 0) {
        sh[warp][RS_NSUM] = vmin;
        sh[warp][RS_NSUM + 1] = vmax;
    }
    __syncthreads();
    if (threadIdx.x < RS_NPART) {
        const int k = threadIdx.x;
        double v = sh[0][k];
        for (int w = 1; w < RS_THREADS / 32; ++w) {
            if (k == RS_NSUM) v = fmin(v, sh[w][k]);
            else if (k == RS_NSUM + 1) v = fmax(v, sh[w][k]);
            else v += sh[w][k];
        }
        part[(size_t)blockIdx.x * RS_NPART + k] = v;
        __threadfence();  // the partial is visible device-wide before this block counts itself in
    }
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(arrivals, 1ull) == (unsigned long long)gridDim.x - 1);
    __syncthreads();
    if (!is_last) return;

    // last block to arrive: fixed-order compensated sum over the blocks, in
    // RS_SEGS contiguous segments, then the segments in order
    __threadfence();
    const int nb = (int)gridDim.x;
    const int per = (nb + RS_SEGS - 1) / RS_SEGS;
    if (threadIdx.x < RS_NPART * RS_SEGS) {
        const int k = threadIdx.x / RS_SEGS, sg = threadIdx.x % RS_SEGS;
        const int b0 = sg * per, b1 = min(nb, b0 + per);
        double s = 0.0, c = 0.0;
        if (k == RS_NSUM) s = INFINITY;
        if (k == RS_NSUM + 1) s = -INFINITY;
        for (int b = b0; b < b1; ++b) {
            const double v = __ldcg(part + (size_t)b * RS_NPART + k);
            if (k == RS_NSUM) s = fmin(s, v);
            else if (k == RS_NSUM + 1) s = fmax(s, v);
            else rs_add(s, c, v);
        }
        seg_s[k][sg] = s;
        seg_c[k][sg] = c;
    }
    __syncthreads();
    if (threadIdx.x < RS_NPART) {
        const int k = threadIdx.x;
        double s = seg_s[k][0], c = seg_c[k][0];
        for (int sg = 1; sg < RS_SEGS; ++sg) {
            if (k == RS_NSUM) s = fmin(s, seg_s[k][sg]);
            else if (k == RS_NSUM + 1) s = fmax(s, seg_s[k][sg]);
            else {
                rs_add(s, c, seg_s[k][sg]);
                c += seg_c[k][sg];
            }
        }
        result[k] = (k >= RS_NSUM) ? s : s + c;
    }
    if (threadIdx.x == 0) atomicExch(arrivals, 0ull);  // ready for the next call
}

// Device address of g_reduce_scratch per device, valid for the context whose
// id it is stored with. The driver's context calls are reached through the
// runtime's entry-point query, so the library needs no link to libcuda.
constexpr int RS_MAX_DEVICES = 64;
struct RsAddr {
    unsigned long long ctx_id;
    double* addr;
};
static RsAddr g_scratch_addr[RS_MAX_DEVICES];
static std::mutex g_scratch_mutex;

typedef CUresult (*RsCtxGetCurrent)(CUcontext*);
typedef CUresult (*RsCtxGetId)(CUcontext, unsigned long long*);

// id of the calling thread's current context (the device's primary context,
// made current by the caller); false when it cannot be read
static bool current_context_id(unsigned long long* id) {
    static RsCtxGetCurrent get_current = nullptr;
    static RsCtxGetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<RsCtxGetCurrent>(fn);
        fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<RsCtxGetId>(fn);
    });
    if (!get_current || !get_id) return false;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

static int scratch_address(dl_handle* h, double** out) {
    if (h->device < 0 || h->device >= RS_MAX_DEVICES)
        return set_error(h, DL_ERR_UNSUPPORTED, "dl_reduce_static supports device ordinals below %d", RS_MAX_DEVICES);
    // the handle's device is current (dl_reduce_static makes it so), and its
    // primary context exists since dl_create
    unsigned long long id = 0;
    const bool have_id = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    RsAddr& c = g_scratch_addr[h->device];
    if (have_id && c.addr && c.ctx_id == id) {
        *out = c.addr;
        return DL_OK;
    }
    void* addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_reduce_scratch);
    if (e != cudaSuccess) return check_cuda(h, e, "cudaGetSymbolAddress(g_reduce_scratch)");
    // without a context id the address is looked up on every call
    c.ctx_id = have_id ? id : 0;
    c.addr = have_id ? static_cast<double*>(addr) : nullptr;
    *out = static_cast<double*>(addr);
    return DL_OK;
}

template <typename T>
static int reduce_static_any(dl_handle* h, const T* d_mac, double phi_off, double p_off, int nblocks, dl_diag* out) {
    double* scratch = nullptr;
    int rc = scratch_address(h, &scratch);
    if (rc != DL_OK) return rc;
    RsArgs a;
    memset(&a, 0, sizeof(a));
    diag_consts(h, phi_off, p_off, a.k);
    // the arrival counter starts at zero whatever an earlier launch left
    DL_CUDA(h, cudaMemsetAsync(scratch + (size_t)RS_MAX_BLOCKS * RS_NPART + RS_NPART, 0, sizeof(unsigned long long),
                               h->stream));
    reduce_static_kernel<T><<<nblocks, RS_THREADS, 0, h->stream>>>(d_mac, a, scratch);
    DL_CUDA(h, cudaGetLastError());
    h->launches += 1;
    double r[RS_NPART];
    DL_CUDA(h, cudaMemcpyAsync(r, scratch + (size_t)RS_MAX_BLOCKS * RS_NPART, sizeof(r), cudaMemcpyDeviceToHost,
                               h->stream));
    DevState st;
    DL_CUDA(h, cudaMemcpyAsync(&st, h->d_state, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    memset(out, 0, sizeof(*out));
    out->phi_sum = r[0];
    out->p_sum = r[1];
    out->mom[0] = r[2];
    out->mom[1] = r[3];
    out->mom[2] = r[4];
    out->ke = r[5];
    out->diss = r[6];
    out->vol_count = r[7];
    out->vol_smooth = r[8];
    out->p_in = r[9];
    out->n_in = r[10];
    out->p_out = r[11];
    out->n_out = r[12];
    out->w_sum = r[13];
    for (int k = 0; k < 3; ++k) out->w_x[k] = r[14 + k];
    for (int k = 0; k < 6; ++k) out->w_xx[k] = r[17 + k];
    out->phi_min = r[RS_NSUM];
    out->phi_max = r[RS_NSUM + 1];
    out->step = h->step;
    out->nan_flag = st.nan_flag;
    return DL_OK;
}

}  // namespace dl

extern "C" int dl_reduce_static(dl_handle* h, int nblocks, dl_diag* out) {
    if (!h || !out) return DL_ERR_ARG;
    if (nblocks == 0) nblocks = dl::RS_DEFAULT_BLOCKS;
    if (nblocks < 1 || nblocks > DL_REDUCE_STATIC_MAX_BLOCKS)
        return dl::set_error(h, DL_ERR_ARG,
                             "dl_reduce_static: nblocks %d is outside 1..%d (the fixed scratch of %d bytes holds the "
                             "partial sums of at most %d blocks); pass 0 for the default of %d",
                             nblocks, DL_REDUCE_STATIC_MAX_BLOCKS, (int)DL_REDUCE_STATIC_SCRATCH_BYTES,
                             DL_REDUCE_STATIC_MAX_BLOCKS, dl::RS_DEFAULT_BLOCKS);
    if (!h->fields_set) return dl::set_error(h, DL_ERR_STATE, "dl_reduce_static: fields not set");
    // a push step's state is settled first (one launch, no allocation)
    if ((h->form == DL_FORM_FP32 || h->form == DL_FORM_FP16) && h->pushed) {
        const int src = dl::fast_settle(h);
        if (src != DL_OK) return src;
    }
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != h->device) {
        const cudaError_t e = cudaSetDevice(h->device);
        if (e != cudaSuccess) return dl::check_cuda(h, e, "cudaSetDevice");
    }
    const bool fast = h->form != DL_FORM_FP64;
    const int rc = fast ? dl::reduce_static_any<float>(h, h->mac32[h->cur], h->P.phi1, 1.0 / 3.0, nblocks, out)
                        : dl::reduce_static_any<double>(h, h->mac64[h->cur], 0.0, 0.0, nblocks, out);
    if (prev >= 0 && prev != h->device) cudaSetDevice(prev);
    return rc;
}
