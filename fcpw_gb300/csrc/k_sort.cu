// Spatial reordering of query batches and record packing for the wide kernels.
//
// Queries are bucketed by a Morton-ordered cell of a 2^18-cell grid (64^3 in
// 3D, 512^2 in 2D) over a box around the scene: a counting sort (histogram,
// exclusive scan, scatter). Threads of a warp then traverse neighbouring
// queries, which keeps their paths through the tree alike. The order inside a
// cell is whatever the scatter's atomics give; results are written back to
// each query's own slot, so the order never shows in the output.
#include "kernels.h"

namespace fcpwgb {

FCPWGB_D uint32_t spread3(uint32_t v) {  // 6 bits -> every third bit
    v &= 0x3fu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
FCPWGB_D uint32_t spread2(uint32_t v) {  // 9 bits -> every second bit
    v &= 0x1ffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

FCPWGB_D uint32_t cellOf(const SortGrid &g, float3 c) {
    if (g.dim == 3) {
        float fx = (c.x - g.lo.x) * g.invCell.x, fy = (c.y - g.lo.y) * g.invCell.y, fz = (c.z - g.lo.z) * g.invCell.z;
        uint32_t ix = (uint32_t)fminf(fmaxf(fx, 0.0f), 63.0f);
        uint32_t iy = (uint32_t)fminf(fmaxf(fy, 0.0f), 63.0f);
        uint32_t iz = (uint32_t)fminf(fmaxf(fz, 0.0f), 63.0f);
        return spread3(ix) | (spread3(iy) << 1) | (spread3(iz) << 2);
    }
    float fx = (c.x - g.lo.x) * g.invCell.x, fy = (c.y - g.lo.y) * g.invCell.y;
    uint32_t ix = (uint32_t)fminf(fmaxf(fx, 0.0f), 511.0f);
    uint32_t iy = (uint32_t)fminf(fmaxf(fy, 0.0f), 511.0f);
    return spread2(ix) | (spread2(iy) << 1);
}

__global__ void kCellHistogram(SortGrid g, const DevSphere *__restrict__ q, uint32_t n, uint32_t *cells) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 s = ldg4(q + i);
    atomicAdd(cells + cellOf(g, make_float3(s.x, s.y, s.z)), 1u);
}

// exclusive scan of 2^18 counters with one block of 1024 threads
__global__ void __launch_bounds__(1024) kScanCells(uint32_t *cells) {
    constexpr uint32_t kCells = 1u << kSortCellBits, kPer = kCells / 1024;
    __shared__ uint32_t part[1024];
    uint32_t t = threadIdx.x, base = t * kPer, sum = 0;
    for (uint32_t k = 0; k < kPer; k++) sum += cells[base + k];
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive scan of the partial sums
        uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
    for (uint32_t k = 0; k < kPer; k++) {
        uint32_t c = cells[base + k];
        cells[base + k] = run;
        run += c;
    }
}

__global__ void kScatterQueries(SortGrid g, const DevSphere *__restrict__ q, uint32_t n, uint32_t *cells,
                                DevSphere *sorted, uint32_t *perm) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 s = ldg4(q + i);
    uint32_t pos = atomicAdd(cells + cellOf(g, make_float3(s.x, s.y, s.z)), 1u);
    reinterpret_cast<float4 *>(sorted)[pos] = s;
    perm[pos] = i;
}

cudaError_t launchSortQueries(const SortGrid &g, const DevSphere *spheres, uint32_t n, uint32_t *cells,
                              DevSphere *sorted, uint32_t *perm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(cells, 0, sizeof(uint32_t) << kSortCellBits, s);
    if (e != cudaSuccess) return e;
    uint32_t blocks = (n + 255) / 256;
    kCellHistogram<<<blocks, 256, 0, s>>>(g, spheres, n, cells);
    kScanCells<<<1, 1024, 0, s>>>(cells);
    kScatterQueries<<<blocks, 256, 0, s>>>(g, spheres, n, cells, sorted, perm);
    return cudaGetLastError();
}

__global__ void kPackTri48(const DevTriangle *__restrict__ t, uint32_t n, float4 *out) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    DevTriangle x = t[k];
    out[3 * k] = make_float4(x.pa.x, x.pa.y, x.pa.z, __uint_as_float(x.index));
    out[3 * k + 1] = make_float4(x.pb.x, x.pb.y, x.pb.z, 0.0f);
    out[3 * k + 2] = make_float4(x.pc.x, x.pc.y, x.pc.z, 0.0f);
}

cudaError_t launchPackTri48(const DevTriangle *tris, uint32_t n, float4 *out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    kPackTri48<<<(n + 255) / 256, 256, 0, s>>>(tris, n, out);
    return cudaGetLastError();
}

}  // namespace fcpwgb
