// labels.cu -- droplet labelling: connected components of the sites with
// phi >= (phi1 + phi2)/2 on the periodic lattice, and their volumes (site
// counts). The reference does this in post-processing with a single-pass
// Hoshen-Kopelman scan (program/percolation.f90:108-259, threshold :112,
// volumes :279-295); that scan only looks back at already-visited sites, so it
// misses joins across the x and y periodic boundaries. Here every periodic
// join is made; the connectivity is selectable and includes the reference's
// neighbour set made symmetric (faces plus the xz and yz edges).
//
// Union-find on the device: parent[s] = s for a foreground site; every site
// unites with the forward half of its neighbour set, linking the larger root
// under the smaller one with atomicCAS (parents only decrease, so every chain
// is finite); then each site points at its root, roots count their sites,
// and roots get compact ids.
#include "dl_internal.cuh"
#include "dl_device.cuh"

#include <algorithm>
#include <string.h>
#include <vector>

namespace dl {

struct LabelArgs {
    int nx, ny, nz;
    int N;
    const double* phi64;  // FP64 form: phi
    const float* dphi32;  // FP32 forms: phi - phi1
    double thr64;         // (phi1 + phi2) / 2
    float thr32;          // (phi2 - phi1) / 2 for dphi
    int* parent;
    int* count;
    int* ids;
    int* vols;
    int* nroots;
    int* err;
    int ndir;
    int3 dirs[13];        // forward half of the neighbour set
};

__device__ __forceinline__ bool fg(const LabelArgs& a, int s) {
    return a.phi64 ? (a.phi64[s] >= a.thr64) : (a.dphi32[s] >= a.thr32);
}

constexpr int LBL_MAXIT = 1 << 24;

__device__ __forceinline__ int find_root(const LabelArgs& a, int x) {
    for (int it = 0; it < LBL_MAXIT; ++it) {
        const int p = __ldcg(a.parent + x);
        if (p == x) return x;
        x = p;
    }
    atomicExch(a.err, 1);
    return x;
}

__global__ void lbl_init(LabelArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    a.parent[s] = fg(a, s) ? s : -1;
    a.count[s] = 0;
}

__global__ void lbl_union(LabelArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N || __ldcg(a.parent + s) < 0) return;
    const int x = s % a.nx, y = (s / a.nx) % a.ny, z = s / (a.nx * a.ny);
    for (int d = 0; d < a.ndir; ++d) {
        const int3 o = a.dirs[d];
        int xx = x + o.x, yy = y + o.y, zz = z + o.z;
        xx = xx < 0 ? xx + a.nx : (xx >= a.nx ? xx - a.nx : xx);
        yy = yy < 0 ? yy + a.ny : (yy >= a.ny ? yy - a.ny : yy);
        zz = zz < 0 ? zz + a.nz : (zz >= a.nz ? zz - a.nz : zz);
        const int t = xx + a.nx * (yy + a.ny * zz);
        if (__ldcg(a.parent + t) < 0) continue;
        int u = s, v = t;
        for (int it = 0; it < LBL_MAXIT; ++it) {
            u = find_root(a, u);
            v = find_root(a, v);
            if (u == v) break;
            if (u < v) {
                const int w = u;
                u = v;
                v = w;
            }
            const int old = atomicCAS(a.parent + u, u, v);
            if (old == u) break;
            u = old;
            if (it == LBL_MAXIT - 1) atomicExch(a.err, 1);
        }
    }
}

__global__ void lbl_compress_count(LabelArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N || a.parent[s] < 0) return;
    const int r = find_root(a, s);
    a.parent[s] = r;
    atomicAdd(a.count + r, 1);
}

__global__ void lbl_compact(LabelArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    if (a.parent[s] == s) {
        const int id = atomicAdd(a.nroots, 1);
        a.ids[s] = id + 1;
        a.vols[id] = a.count[s];
    }
}

__global__ void lbl_final(LabelArgs a, int* out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    const int r = a.parent[s];
    out[s] = r < 0 ? 0 : a.ids[r];
}

static void directions(int conn, LabelArgs& a) {
    // forward half: (dz > 0) or (dz == 0 and dy > 0) or (dz == 0 and dy == 0 and dx > 0)
    a.ndir = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const bool fwd = dz > 0 || (dz == 0 && dy > 0) || (dz == 0 && dy == 0 && dx > 0);
                if (!fwd) continue;
                const int nnz = (dx != 0) + (dy != 0) + (dz != 0);
                bool use = false;
                if (conn == 6) use = nnz == 1;
                else if (conn == 18) use = nnz <= 2;
                else if (conn == 26) use = true;
                else if (conn == 14) use = nnz == 1 || (nnz == 2 && dz != 0);  // faces + xz and yz edges
                if (use) a.dirs[a.ndir++] = make_int3(dx, dy, dz);
            }
}

int label_droplets(dl_handle* h, int conn, int* labels_host, long long* ndrops, double* volumes, long long maxv) {
    if (conn != 6 && conn != 14 && conn != 18 && conn != 26)
        return set_error(h, DL_ERR_ARG, "connectivity must be 6, 14, 18 or 26");
    if (h->N > (size_t)0x7fffffff) return set_error(h, DL_ERR_UNSUPPORTED, "labelling supports < 2^31 sites");
    const int N = (int)h->N;
    if (!h->lbl_buf) DL_CUDA(h, cudaMalloc(&h->lbl_buf, sizeof(int) * (4 * (size_t)N + 2)));
    LabelArgs a;
    memset(&a, 0, sizeof(a));
    a.nx = h->nx;
    a.ny = h->ny;
    a.nz = h->nz;
    a.N = N;
    if (h->form == DL_FORM_FP64) {
        a.phi64 = h->mac64[h->cur];
        a.thr64 = (h->P.phi1 + h->P.phi2) / 2.0;
    } else {
        a.dphi32 = h->mac32[h->cur];
        a.thr32 = (float)((h->P.phi2 - h->P.phi1) / 2.0);
    }
    a.parent = h->lbl_buf;
    a.count = a.parent + N;
    a.ids = a.count + N;
    a.vols = a.ids + N;
    a.nroots = a.vols + N;
    a.err = a.nroots + 1;
    directions(conn, a);
    DL_CUDA(h, cudaMemsetAsync(a.nroots, 0, 2 * sizeof(int), h->stream));
    const unsigned nb = (unsigned)((N + 255) / 256);
    DL_LAUNCH(h, false, (lbl_init<<<nb, 256, 0, h->stream>>>(a)));
    DL_LAUNCH(h, false, (lbl_union<<<nb, 256, 0, h->stream>>>(a)));
    DL_LAUNCH(h, false, (lbl_compress_count<<<nb, 256, 0, h->stream>>>(a)));
    DL_LAUNCH(h, false, (lbl_compact<<<nb, 256, 0, h->stream>>>(a)));
    DL_CUDA(h, cudaGetLastError());
    int hdr[2];
    DL_CUDA(h, cudaMemcpyAsync(hdr, a.nroots, sizeof(hdr), cudaMemcpyDeviceToHost, h->stream));
    DL_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hdr[1]) return set_error(h, DL_ERR_TIMEOUT, "labelling union-find exceeded its iteration bound");
    const int n = hdr[0];
    std::vector<int> vols((size_t)n);
    if (n) DL_CUDA(h, cudaMemcpy(vols.data(), a.vols, sizeof(int) * n, cudaMemcpyDeviceToHost));
    // order by decreasing volume (ties by id)
    std::vector<int> order((size_t)n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return vols[p] > vols[q]; });
    *ndrops = n;
    for (long long i = 0; i < n && i < maxv; ++i) volumes[i] = (double)vols[order[i]];
    if (labels_host) {
        DL_LAUNCH(h, false, (lbl_final<<<nb, 256, 0, h->stream>>>(a, a.count)));
        DL_CUDA(h, cudaMemcpyAsync(labels_host, a.count, sizeof(int) * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
        DL_CUDA(h, cudaStreamSynchronize(h->stream));
        std::vector<int> rank((size_t)n + 1, 0);
        for (int i = 0; i < n; ++i) rank[order[i] + 1] = i + 1;
        for (int s = 0; s < N; ++s) labels_host[s] = rank[labels_host[s]];
    }
    return DL_OK;
}

}  // namespace dl
