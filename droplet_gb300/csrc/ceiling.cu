// ceiling.cu -- measured ceilings beside the roofline.
// dl_pull_ceiling: the memory ceiling of the step's access
// pattern on this GPU. A z-marching 32 x 8 column kernel pulls the 15
// direction arrays of g from x - c_i (periodic) and writes them to the other
// buffer, with no collision: what the fused step's loads and stores cost
// without its arithmetic. It runs on the handle's own g buffers (the
// next-step buffer is overwritten, the current one is only read) and is
// timed with CUDA events on the handle's stream.
// dl_fp64_ceiling: FP64 FMA throughput of this GPU (the bound of the plain
// FP64 form), from independent FMA chains on every SM.
#include "dl_internal.cuh"

#include <cuda_fp16.h>

namespace dl {

constexpr int CL_LZ = 32;

__device__ __forceinline__ int cl_wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

template <typename T>
__global__ void __launch_bounds__(256, 2) pull_copy(const T* __restrict__ in, T* __restrict__ out, int nx, int ny,
                                                    int nz) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const size_t N = (size_t)nx * ny * nz;
    const int z0 = blockIdx.z * CL_LZ, z1 = min(z0 + CL_LZ, nz);
    for (int z = z0; z < z1; ++z) {
        const size_t d = x + (size_t)nx * (y + (size_t)ny * z);
        T v[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const size_t s = cl_wrap(x - cx(i), nx) + (size_t)nx * (cl_wrap(y - cy(i), ny) + (size_t)ny * cl_wrap(z - cz(i), nz));
            v[i] = __ldg(in + i * N + s);
        }
#pragma unroll
        for (int i = 0; i < Q; ++i) out[i * N + d] = v[i];
    }
}

int pull_ceiling(dl_handle* h, int repeats, double* gbps) {
    if (h->form == DL_FORM_FP64) return set_error(h, DL_ERR_UNSUPPORTED, "dl_pull_ceiling is for the FP32 and FP16 forms");
    if (repeats < 1) return set_error(h, DL_ERR_ARG, "repeats must be >= 1");
    const dim3 grid((h->nx + 31) / 32, (h->ny + 7) / 8, (h->nz + CL_LZ - 1) / CL_LZ), block(32, 8);
    const bool half = h->form == DL_FORM_FP16;
    const void* in = h->gs[h->cur];
    void* out = h->gs[1 - h->cur];
    auto launch = [&]() {
        if (half) pull_copy<__half><<<grid, block, 0, h->stream>>>((const __half*)in, (__half*)out, h->nx, h->ny, h->nz);
        else pull_copy<float><<<grid, block, 0, h->stream>>>((const float*)in, (float*)out, h->nx, h->ny, h->nz);
        h->launches += 1;
    };
    launch();  // warm-up
    cudaEvent_t e0, e1;
    DL_CUDA(h, cudaEventCreate(&e0));
    DL_CUDA(h, cudaEventCreate(&e1));
    cudaEventRecord(e0, h->stream);
    for (int r = 0; r < repeats; ++r) launch();
    cudaEventRecord(e1, h->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    DL_CUDA(h, e);
    DL_CUDA(h, cudaGetLastError());
    const double bytes = 2.0 * Q * (half ? 2.0 : 4.0) * (double)h->N;
    *gbps = bytes / ((double)ms / repeats * 1e-3) / 1e9;
    return DL_OK;
}

// FP64 FMA throughput: 8 independent chains per thread, 4 blocks per SM
__global__ void __launch_bounds__(256) fma64_loop(double* out, int iters, double a, double b) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = (double)(threadIdx.x + k) * 1e-3;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = fma(v[k], a, b);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += v[k];
    if (out && s == 12345.6789) out[0] = s;  // keeps the chains live (out is null)
}

int fp64_ceiling(dl_handle* h, double* tflops) {
    int sms = 0;
    DL_CUDA(h, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
    const int blocks = 4 * sms, iters = 4096;
    double* sink = nullptr;
    fma64_loop<<<blocks, 256, 0, h->stream>>>(sink, iters, 0.999999, 1e-7);  // warm-up
    cudaEvent_t e0, e1;
    DL_CUDA(h, cudaEventCreate(&e0));
    DL_CUDA(h, cudaEventCreate(&e1));
    cudaEventRecord(e0, h->stream);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) fma64_loop<<<blocks, 256, 0, h->stream>>>(sink, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, h->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    DL_CUDA(h, e);
    DL_CUDA(h, cudaGetLastError());
    h->launches += reps + 1;
    const double flops = 2.0 * 8.0 * iters * 256.0 * blocks * reps;
    *tflops = flops / ((double)ms * 1e-3) / 1e12;
    return DL_OK;
}

}  // namespace dl
