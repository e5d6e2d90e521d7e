// Spatial reordering of query batches and record packing for the wide kernels.
//
// Queries (sphere centres, ray origins) are bucketed by a Morton-ordered cell of a 2^18-cell grid (64^3 in
// 3D, 512^2 in 2D) and counting-sorted (histogram, exclusive scan, scatter).
// The grid spans the bounding box of the batch's own query centres, clipped
// to limits around the scene, so that cells are neither empty nor crowded
// whatever the query distribution. Threads of a warp then traverse
// neighbouring queries, which keeps their paths through the tree alike. The
// order inside a cell is whatever the scatter's atomics give; results are
// written back to each query's own slot, so the order never shows in the
// output.
#include <algorithm>

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

// float <-> int with the same order, so bounds reduce with integer atomics
FCPWGB_D int orderedInt(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
FCPWGB_D float orderedFloat(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

struct CellGrid {
    float3 lo, inv;
};

// qb: ordered-int min[3], max[3] of the query centres
FCPWGB_D CellGrid cellGrid(const SortLimits &lim, const int *qb) {
    const float cells = lim.dim == 3 ? 64.0f : 512.0f;
    float lo[3] = {lim.lo.x, lim.lo.y, lim.lo.z}, hi[3] = {lim.hi.x, lim.hi.y, lim.hi.z}, inv[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float ql = orderedFloat(__ldg(qb + a)), qh = orderedFloat(__ldg(qb + 3 + a));
        float l = fmaxf(ql, lo[a]), h = fminf(qh, hi[a]);
        if (!(h > l)) {  // no spread on this axis (or no finite query): one cell layer
            l = fminf(fmaxf(ql, lo[a]), hi[a]);
            h = l;
        }
        lo[a] = l;
        inv[a] = cells / fmaxf(h - l, 1e-20f);
    }
    CellGrid g;
    g.lo = make_float3(lo[0], lo[1], lo[2]);
    g.inv = make_float3(inv[0], inv[1], inv[2]);
    return g;
}

FCPWGB_D uint32_t cellOf(int dim, const CellGrid &g, float3 c) {
    if (dim == 3) {
        float fx = (c.x - g.lo.x) * g.inv.x, fy = (c.y - g.lo.y) * g.inv.y, fz = (c.z - g.lo.z) * g.inv.z;
        uint32_t ix = (uint32_t)fminf(fmaxf(fx, 0.0f), 63.0f);
        uint32_t iy = (uint32_t)fminf(fmaxf(fy, 0.0f), 63.0f);
        uint32_t iz = (uint32_t)fminf(fmaxf(fz, 0.0f), 63.0f);
        return spread3(ix) | (spread3(iy) << 1) | (spread3(iz) << 2);
    }
    float fx = (c.x - g.lo.x) * g.inv.x, fy = (c.y - g.lo.y) * g.inv.y;
    uint32_t ix = (uint32_t)fminf(fmaxf(fx, 0.0f), 511.0f);
    uint32_t iy = (uint32_t)fminf(fmaxf(fy, 0.0f), 511.0f);
    return spread2(ix) | (spread2(iy) << 1);
}

// the position a record is sorted by: a sphere's centre, a ray's origin
FCPWGB_D float3 recordPosition(const DevSphere *q, uint32_t i) {
    float4 s = ldg4(q + i);
    return make_float3(s.x, s.y, s.z);
}
FCPWGB_D float3 recordPosition(const DevRay *q, uint32_t i) {  // 40 B records: 8 B aligned
    const unsigned char *p = reinterpret_cast<const unsigned char *>(q + i);
    float2 a = ldg2(p), b = ldg2(p + 8);
    return make_float3(a.x, a.y, b.x);
}
FCPWGB_D void copyRecord(const DevSphere *q, uint32_t i, DevSphere *dst, uint32_t j) {
    reinterpret_cast<float4 *>(dst)[j] = ldg4(q + i);
}
FCPWGB_D void copyRecord(const DevRay *q, uint32_t i, DevRay *dst, uint32_t j) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(q + i);
    float2 *d = reinterpret_cast<float2 *>(dst + j);
#pragma unroll
    for (int k = 0; k < 5; k++) d[k] = ldg2(p + 8 * k);
}

// min/max of the finite record positions: a warp reduction, then one atomic
// per warp and axis into qb (initialised to +3.4e38 / -3.4e38 by a byte memset)
template<class Rec> __global__ void kQueryBounds(const Rec *__restrict__ q, uint32_t n, int *qb) {
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float3 s = recordPosition(q, i);
        float v[3] = {s.x, s.y, s.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (isfinite(v[a])) {
                lo[a] = fminf(lo[a], v[a]);
                hi[a] = fmaxf(hi[a], v[a]);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    if ((threadIdx.x & 31u) == 0) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            atomicMin(qb + a, orderedInt(lo[a]));
            atomicMax(qb + 3 + a, orderedInt(hi[a]));
        }
    }
}

template<class Rec>
__global__ void kCellHistogram(SortLimits lim, const int *qb, const Rec *__restrict__ q, uint32_t n,
                               uint32_t *cells) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    CellGrid g = cellGrid(lim, qb);
    atomicAdd(cells + cellOf(lim.dim, g, recordPosition(q, i)), 1u);
}

template<class Rec>
__global__ void kScatterQueries(SortLimits lim, const int *qb, const Rec *__restrict__ q, uint32_t n,
                                uint32_t *cells, Rec *sorted, uint32_t *perm) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    CellGrid g = cellGrid(lim, qb);
    uint32_t pos = atomicAdd(cells + cellOf(lim.dim, g, recordPosition(q, i)), 1u);
    copyRecord(q, i, sorted, pos);
    perm[pos] = i;
}

cudaError_t scanCounts(uint32_t *cells, uint32_t nCells, uint32_t *tileSums, cudaStream_t s);

template<class Rec>
cudaError_t sortRecords(const SortLimits &lim, const Rec *recs, uint32_t n, uint32_t *cells, Rec *sorted,
                        uint32_t *perm, int numSMs, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    int *qb = reinterpret_cast<int *>(cells + kSortCells);
    cudaError_t e = cudaMemsetAsync(cells, 0, sizeof(uint32_t) * kSortCells, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(qb, 0x7f, 3 * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(qb + 3, 0x80, 3 * sizeof(int), s);
    if (e != cudaSuccess) return e;
    uint32_t blocks = (n + 255) / 256;
    kQueryBounds<Rec><<<std::min<uint32_t>(blocks, (uint32_t)std::max(numSMs, 1) * 8u), 256, 0, s>>>(recs, n, qb);
    kCellHistogram<Rec><<<blocks, 256, 0, s>>>(lim, qb, recs, n, cells);
    if ((e = scanCounts(cells, kSortCells, cells + kSortCells + 8, s)) != cudaSuccess) return e;
    kScatterQueries<Rec><<<blocks, 256, 0, s>>>(lim, qb, recs, n, cells, sorted, perm);
    return cudaGetLastError();
}

cudaError_t launchSortQueries(const SortLimits &lim, const DevSphere *spheres, uint32_t n, uint32_t *cells,
                              DevSphere *sorted, uint32_t *perm, int numSMs, cudaStream_t s) {
    return sortRecords(lim, spheres, n, cells, sorted, perm, numSMs, s);
}

cudaError_t launchSortRays(const SortLimits &lim, const DevRay *rays, uint32_t n, uint32_t *cells, DevRay *sorted,
                           uint32_t *perm, int numSMs, cudaStream_t s) {
    return sortRecords(lim, rays, n, cells, sorted, perm, numSMs, s);
}

// ---------------------------------------------------------------- batches
// Queries of many scenes, grouped by scene (offsets[s] .. offsets[s+1]), are
// ordered by (scene, Morton cell of that scene's own grid): one counting sort
// over the concatenated cell ranges of all scenes.

// scene of query i: the last s with offsets[s] <= i (empty scenes are skipped)
FCPWGB_D uint32_t sceneOf(const uint32_t *__restrict__ offsets, uint32_t nScenes, uint32_t i) {
    uint32_t lo = 0, hi = nScenes;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(offsets + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

FCPWGB_D uint32_t batchCell(int dim, const BatchSceneGrid &g, float3 c) {
    const float top = (float)((1u << g.bits) - 1u);
    uint32_t ix = (uint32_t)fminf(fmaxf((c.x - g.lo.x) * g.inv.x, 0.0f), top);
    uint32_t iy = (uint32_t)fminf(fmaxf((c.y - g.lo.y) * g.inv.y, 0.0f), top);
    if (dim == 3) {
        uint32_t iz = (uint32_t)fminf(fmaxf((c.z - g.lo.z) * g.inv.z, 0.0f), top);
        return g.cellBase + (spread3(ix) | (spread3(iy) << 1) | (spread3(iz) << 2));
    }
    return g.cellBase + (spread2(ix) | (spread2(iy) << 1));
}

__global__ void kBatchHistogram(int dim, const BatchSceneGrid *__restrict__ grids, const uint32_t *__restrict__ offsets,
                                uint32_t nScenes, const DevSphere *__restrict__ q, uint32_t n, uint32_t *cells) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BatchSceneGrid g = grids[sceneOf(offsets, nScenes, i)];
    float4 s = ldg4(q + i);
    atomicAdd(cells + batchCell(dim, g, make_float3(s.x, s.y, s.z)), 1u);
}

// exclusive scan of counters: tiles of 4096 scanned in place (tile totals to
// sums), the totals scanned by one block, then added back
constexpr uint32_t kScanTile = 4096;
__global__ void __launch_bounds__(1024) kScanTiles(uint32_t *cells, uint32_t nCells, uint32_t *sums) {
    __shared__ uint32_t part[1024];
    uint32_t t = threadIdx.x, base = blockIdx.x * kScanTile + t * 4;
    uint32_t v[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = base + k < nCells ? cells[base + k] : 0u;
        sum += v[k];
    }
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {
        uint32_t x = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (base + k < nCells) cells[base + k] = run;
        run += v[k];
    }
    if (t == 1023) sums[blockIdx.x] = part[1023];
}

__global__ void __launch_bounds__(1024) kScanTileSums(uint32_t *sums, uint32_t nTiles) {
    __shared__ uint32_t part[1024];
    uint32_t t = threadIdx.x, per = (nTiles + 1023) / 1024, base = t * per, sum = 0;
    for (uint32_t k = 0; k < per; k++)
        if (base + k < nTiles) sum += sums[base + k];
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {
        uint32_t x = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
    for (uint32_t k = 0; k < per; k++) {
        if (base + k < nTiles) {
            uint32_t c = sums[base + k];
            sums[base + k] = run;
            run += c;
        }
    }
}

__global__ void kAddTileBase(uint32_t *cells, uint32_t nCells, const uint32_t *sums) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nCells) cells[i] += sums[i / kScanTile];
}

__global__ void kBatchScatter(int dim, const BatchSceneGrid *__restrict__ grids, const uint32_t *__restrict__ offsets,
                              uint32_t nScenes, const DevSphere *__restrict__ q, uint32_t n, uint32_t *cells,
                              DevSphere *sorted, uint32_t *perm, uint32_t *roots) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BatchSceneGrid g = grids[sceneOf(offsets, nScenes, i)];
    float4 s = ldg4(q + i);
    uint32_t pos = atomicAdd(cells + batchCell(dim, g, make_float3(s.x, s.y, s.z)), 1u);
    reinterpret_cast<float4 *>(sorted)[pos] = s;
    perm[pos] = i;
    roots[pos] = g.root;
}

uint32_t batchScanTiles(uint32_t nCells) { return (nCells + kScanTile - 1) / kScanTile; }

// exclusive scan of nCells counters in place; tileSums holds batchScanTiles(nCells) words
cudaError_t scanCounts(uint32_t *cells, uint32_t nCells, uint32_t *tileSums, cudaStream_t s) {
    uint32_t tiles = batchScanTiles(nCells);
    kScanTiles<<<tiles, 1024, 0, s>>>(cells, nCells, tileSums);
    kScanTileSums<<<1, 1024, 0, s>>>(tileSums, tiles);
    kAddTileBase<<<(nCells + 255) / 256, 256, 0, s>>>(cells, nCells, tileSums);
    return cudaGetLastError();
}

cudaError_t launchSortBatchQueries(int dim, const BatchSceneGrid *grids, const uint32_t *offsets, uint32_t nScenes,
                                   const DevSphere *spheres, uint32_t n, uint32_t *cells, uint32_t nCells,
                                   uint32_t *tileSums, DevSphere *sorted, uint32_t *perm, uint32_t *roots,
                                   cudaStream_t s) {
    if (n == 0 || nCells == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(cells, 0, sizeof(uint32_t) * nCells, s);
    if (e != cudaSuccess) return e;
    uint32_t blocks = (n + 255) / 256;
    kBatchHistogram<<<blocks, 256, 0, s>>>(dim, grids, offsets, nScenes, spheres, n, cells);
    if ((e = scanCounts(cells, nCells, tileSums, s)) != cudaSuccess) return e;
    kBatchScatter<<<blocks, 256, 0, s>>>(dim, grids, offsets, nScenes, spheres, n, cells, sorted, perm, roots);
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
