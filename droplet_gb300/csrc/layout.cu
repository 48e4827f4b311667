// layout.cu -- conversion between the device layout of the populations
// (structure of arrays, f[i][z][y][x]) and the reference's host layout
// f_procs(1:15,x,y,z) (direction index fastest), used for checkpoints
// (outputfg, program/lbm_drop_xy.f90:721-743) and for resume / precursor reads
// (program/lbm_drop_xy.f90:789-823).
#include "dl_internal.cuh"

namespace dl {

__global__ void soa_to_aos_kernel(const double* __restrict__ soa, double* __restrict__ aos, long long N) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)Q * N) return;
    const long long s = t / Q;
    const int i = (int)(t - s * Q);
    aos[t] = soa[i * N + s];
}

__global__ void aos_to_soa_kernel(const double* __restrict__ aos, double* __restrict__ soa, long long N) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)Q * N) return;
    const int i = (int)(t / N);
    const long long s = t - i * N;
    soa[t] = aos[s * Q + i];
}

int soa_to_aos(dl_handle* h, const double* d_soa, double* d_aos) {
    const long long n = (long long)Q * h->N;
    DL_LAUNCH(h, false, soa_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(d_soa, d_aos, (long long)h->N));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

int aos_to_soa(dl_handle* h, const double* d_aos, double* d_soa) {
    const long long n = (long long)Q * h->N;
    DL_LAUNCH(h, false, aos_to_soa_kernel<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(d_aos, d_soa, (long long)h->N));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

__global__ void fill_kernel(double* __restrict__ d, double v, long long n) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) d[t] = v;
}

int fill_doubles(dl_handle* h, double* d, double v, size_t n) {
    if (n == 0) return DL_OK;
    DL_LAUNCH(h, false, fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(d, v, (long long)n));
    DL_CUDA(h, cudaGetLastError());
    return DL_OK;
}

}  // namespace dl
