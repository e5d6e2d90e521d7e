// Spatial reordering of query batches and record packing for the wide kernels.
//
// Queries (sphere centres, ray origins) are bucketed by the Hilbert index of their cell in a 128^3 grid in 3D
// (512^2 in 2D) and counting-sorted (histogram, exclusive scan, scatter). On 4M queries the 3D grid at 128^3
// made the closest-point packets 1.3 % faster than at 64^3; in 2D 1024^2 was 4 % slower than 512^2 on 8M
// queries. Hilbert order keeps every run of consecutive cells face-connected, where Morton (Z) order jumps
// between blocks: a packet of 32 sorted queries then spans a more compact region (4M queries on the torus,
// 2 queries per cell: 6.01 against 6.39 ms per call; 1M queries on the icosphere, half a query per cell:
// 0.785 against 0.930 ms, 10 % fewer triangle loads per packet).
// The grid spans the bounding box of the batch's own query centres, clipped
// to limits around the scene, so that cells are neither empty nor crowded
// whatever the query distribution. Threads of a warp then traverse
// neighbouring queries, which keeps their paths through the tree alike. The
// order inside a cell is whatever the scatter's atomics give; results are
// written back to each query's own slot, and the wide kernels break exact
// distance ties by primitive index, so the order never shows in the output.
//
// The stable radix sort further down orders the Morton codes of the GPU BVH
// build, where equal codes must keep primitive order.
#include <algorithm>
#include <type_traits>

#include "kernels.h"

namespace fcpwgb {

FCPWGB_D uint32_t spread3(uint32_t v) {  // up to 8 bits -> every third bit
    v &= 0xffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
FCPWGB_D uint32_t spread2(uint32_t v) {  // up to 16 bits -> every second bit
    v &= 0xffffu;
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
    const float cells = lim.dim == 3 ? 128.0f : 512.0f;
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

// Hilbert index of cell coordinates x[0..N-1] of B bits each: J. Skilling,
// "Programming the Hilbert curve", AIP Conf. Proc. 707 (2004) -- the
// coordinates are transformed in place into the curve's "transpose" form
// (inverse undo of the rotations and reflections, then Gray encoding), whose
// bits interleaved, x[0] most significant, are the index. Consecutive indices
// are face-adjacent cells, and the index's top bits are the index of the
// parent cell at half the resolution.
template<int N> FCPWGB_D void hilbertTranspose(uint32_t (&x)[N], int bits) {
    if (bits <= 0) return;
    const uint32_t m = 1u << (bits - 1);
    for (uint32_t q = m; q > 1; q >>= 1) {
        const uint32_t p = q - 1;
#pragma unroll
        for (int i = 0; i < N; i++) {
            if (x[i] & q) {
                x[0] ^= p;
            } else {
                const uint32_t t = (x[0] ^ x[i]) & p;
                x[0] ^= t;
                x[i] ^= t;
            }
        }
    }
#pragma unroll
    for (int i = 1; i < N; i++) x[i] ^= x[i - 1];
    uint32_t t = 0;
    for (uint32_t q = m; q > 1; q >>= 1)
        if (x[N - 1] & q) t ^= q - 1;
#pragma unroll
    for (int i = 0; i < N; i++) x[i] ^= t;
}

FCPWGB_D uint32_t cellOf(int dim, const CellGrid &g, float3 c) {
    if (dim == 3) {
        float fx = (c.x - g.lo.x) * g.inv.x, fy = (c.y - g.lo.y) * g.inv.y, fz = (c.z - g.lo.z) * g.inv.z;
        uint32_t x[3] = {(uint32_t)fminf(fmaxf(fx, 0.0f), 127.0f), (uint32_t)fminf(fmaxf(fy, 0.0f), 127.0f),
                         (uint32_t)fminf(fmaxf(fz, 0.0f), 127.0f)};
        hilbertTranspose<3>(x, 7);
        return (spread3(x[0]) << 2) | (spread3(x[1]) << 1) | spread3(x[2]);
    }
    float fx = (c.x - g.lo.x) * g.inv.x, fy = (c.y - g.lo.y) * g.inv.y;
    uint32_t x[2] = {(uint32_t)fminf(fmaxf(fx, 0.0f), 511.0f), (uint32_t)fminf(fmaxf(fy, 0.0f), 511.0f)};
    hilbertTranspose<2>(x, 9);
    return (spread2(x[0]) << 1) | spread2(x[1]);
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
// the sort cell of a record: a sphere by its centre; a ray by the octant of
// its direction first (the rays of a warp then share their near-child
// order), then the Hilbert index of its origin's cell on a grid half as fine
// per axis (64^3 in 3D, 256^2 in 2D: the index's top bits), so that both fit
// the cells of a sphere grid
FCPWGB_D uint32_t recordCell(int dim, const CellGrid &g, const DevSphere *q, uint32_t i, bool, uint32_t) {
    return cellOf(dim, g, recordPosition(q, i));
}
// inOrder: the caller's rays are already coherent (see kRayCoherence); they
// keep their order, in cells of 32 consecutive rays (nCells bounds the cell)
FCPWGB_D uint32_t recordCell(int dim, const CellGrid &g, const DevRay *q, uint32_t i, bool inOrder,
                             uint32_t nCells) {
    if (inOrder) return min(i >> 5, nCells - 1);
    const unsigned char *p = reinterpret_cast<const unsigned char *>(q + i);
    const float2 a = ldg2(p), b = ldg2(p + 8), c = ldg2(p + 16);  // (o.x, o.y), (o.z, d.x), (d.y, d.z)
    const uint32_t oct = (b.y < 0.0f ? 1u : 0u) | (c.x < 0.0f ? 2u : 0u) | (dim == 3 && c.y < 0.0f ? 4u : 0u);
    if (dim == 3) {
        const uint32_t m = cellOf(3, g, make_float3(a.x, a.y, b.x));  // 21 bits
        return (oct << 18) | (m >> 3);                                 // the parent cell, half as fine
    }
    const uint32_t m = cellOf(2, g, make_float3(a.x, a.y, 0.0f));     // 18 bits
    return (oct << 16) | (m >> 2);
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

// min/max of the finite record positions: four independent loads in flight
// per thread, a warp and then a block reduction, one atomic per block and
// axis into qb (initialised to +3.4e38 / -3.4e38 by a byte memset)
FCPWGB_D void boundsAdd(float3 s, float (&lo)[3], float (&hi)[3]) {
    float v[3] = {s.x, s.y, s.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (isfinite(v[a])) {
            lo[a] = fminf(lo[a], v[a]);
            hi[a] = fmaxf(hi[a], v[a]);
        }
    }
}

constexpr uint32_t kBoundsBlock = 256;
template<class Rec> __global__ void __launch_bounds__(kBoundsBlock) kQueryBounds(const Rec *__restrict__ q, uint32_t n,
                                                                              int *qb) {
    __shared__ float sLo[kBoundsBlock / 32][3], sHi[kBoundsBlock / 32][3];
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    const uint32_t stride = gridDim.x * kBoundsBlock;
    uint32_t i = blockIdx.x * kBoundsBlock + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        float3 s0 = recordPosition(q, i), s1 = recordPosition(q, i + stride);
        float3 s2 = recordPosition(q, i + 2 * stride), s3 = recordPosition(q, i + 3 * stride);
        boundsAdd(s0, lo, hi);
        boundsAdd(s1, lo, hi);
        boundsAdd(s2, lo, hi);
        boundsAdd(s3, lo, hi);
    }
    for (; i < n; i += stride) boundsAdd(recordPosition(q, i), lo, hi);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; a++) {
            sLo[warp][a] = lo[a];
            sHi[warp][a] = hi[a];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        float l = sLo[0][a], h = sHi[0][a];
        for (uint32_t w = 1; w < kBoundsBlock / 32; w++) {
            l = fminf(l, sLo[w][a]);
            h = fmaxf(h, sHi[w][a]);
        }
        atomicMin(qb + a, orderedInt(l));
        atomicMax(qb + 3 + a, orderedInt(h));
    }
}

// qb[6]: how many sampled consecutive pairs of rays point alike (kRayCoherence,
// keepOrder); coherent rays keep the caller's order, and with skipInOrder set
// the caller reads its own array (no sorted copy or permutation is written)
template<class Rec>
__global__ void kCellHistogram(SortLimits lim, const int *qb, const Rec *__restrict__ q, uint32_t n,
                               uint32_t *cells, uint32_t nCells, bool skipInOrder) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool inOrder = keepOrder(qb, n);
    if (inOrder && skipInOrder) return;
    CellGrid g = cellGrid(lim, qb);
    atomicAdd(cells + recordCell(lim.dim, g, q, i, inOrder, nCells), 1u);
}

template<class Rec>
__global__ void kScatterQueries(SortLimits lim, const int *qb, const Rec *__restrict__ q, uint32_t n,
                                uint32_t *cells, uint32_t nCells, Rec *sorted, uint32_t *perm, uint32_t *inv,
                                bool skipInOrder) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool inOrder = keepOrder(qb, n);
    if (inOrder && skipInOrder) return;
    CellGrid g = cellGrid(lim, qb);
    uint32_t pos = atomicAdd(cells + recordCell(lim.dim, g, q, i, inOrder, nCells), 1u);
    copyRecord(q, i, sorted, pos);
    perm[pos] = i;
    if (inv) inv[i] = pos;
}

cudaError_t scanCounts(uint32_t *cells, uint32_t nCells, uint32_t *tileSums, cudaStream_t s);

// Whether the caller's rays are already coherent (camera rays of pixel
// blocks, all from one eye): for up to kCoherenceSamples evenly spaced
// consecutive pairs, counts into qb[6] those whose directions agree (cosine
// > 0.999). With 90 % of them alike the sort keeps the caller's order: a
// spatial sort would put rays of one origin into one cell in arbitrary order
// (measured 3.6 ms against 0.5 ms for 4M camera rays).
__global__ void kRayCoherence(const DevRay *__restrict__ q, uint32_t n, int *qb) {
    const uint32_t samples = min(n > 0 ? n - 1 : 0u, kCoherenceSamples);
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= samples) return;
    const uint32_t i = (uint32_t)(((uint64_t)k * (n - 1)) / samples);
    const unsigned char *p = reinterpret_cast<const unsigned char *>(q + i), *r = p + sizeof(DevRay);
    const float2 a = ldg2(p + 8), b = ldg2(p + 16), c = ldg2(r + 8), d = ldg2(r + 16);  // (o.z, d.x), (d.y, d.z)
    const float dot = a.y * c.y + b.x * d.x + b.y * d.y;
    if (dot > 0.999f) atomicAdd(qb + 6, 1);
}

template<class Rec>
cudaError_t sortRecords(const SortLimits &lim, const Rec *recs, uint32_t n, uint32_t *cells, Rec *sorted,
                        uint32_t *perm, int numSMs, cudaStream_t s, bool skipInOrder = false, uint32_t *inv = nullptr) {
    if (n == 0) return cudaSuccess;
    int *qb = reinterpret_cast<int *>(cells + kSortCells);
    const uint32_t nCells = lim.dim == 3 ? 1u << 21 : 1u << 18;  // the cells cellOf can return
    cudaError_t e = cudaMemsetAsync(cells, 0, sizeof(uint32_t) * nCells, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(qb, 0x7f, 3 * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(qb + 3, 0x80, 3 * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(qb + 6, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    uint32_t blocks = (n + 255) / 256;
    if (std::is_same<Rec, DevRay>::value && n > 1)
        kRayCoherence<<<(std::min(n - 1, kCoherenceSamples) + 255) / 256, 256, 0, s>>>(
            reinterpret_cast<const DevRay *>(recs), n, qb);
    kQueryBounds<Rec><<<std::min<uint32_t>(blocks, (uint32_t)std::max(numSMs, 1) * 8u), kBoundsBlock, 0, s>>>(recs, n,
                                                                                                     qb);
    kCellHistogram<Rec><<<blocks, 256, 0, s>>>(lim, qb, recs, n, cells, nCells, skipInOrder);
    if ((e = scanCounts(cells, nCells, cells + kSortCells + 8, s)) != cudaSuccess) return e;
    kScatterQueries<Rec><<<blocks, 256, 0, s>>>(lim, qb, recs, n, cells, nCells, sorted, perm, inv, skipInOrder);
    return cudaGetLastError();
}

cudaError_t launchSortQueries(const SortLimits &lim, const DevSphere *spheres, uint32_t n, uint32_t *cells,
                              DevSphere *sorted, uint32_t *perm, int numSMs, cudaStream_t s, uint32_t *inv) {
    return sortRecords(lim, spheres, n, cells, sorted, perm, numSMs, s, false, inv);
}

cudaError_t launchSortRays(const SortLimits &lim, const DevRay *rays, uint32_t n, uint32_t *cells, DevRay *sorted,
                           uint32_t *perm, int numSMs, cudaStream_t s, bool skipInOrder) {
    return sortRecords(lim, rays, n, cells, sorted, perm, numSMs, s, skipInOrder);
}

// ---------------------------------------------------------------- batches
// Queries of many scenes, grouped by scene (offsets[s] .. offsets[s+1]), are
// ordered by (scene, Hilbert index of the cell in that scene's own grid): one counting sort
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
        uint32_t x[3] = {ix, iy, (uint32_t)fminf(fmaxf((c.z - g.lo.z) * g.inv.z, 0.0f), top)};
        hilbertTranspose<3>(x, (int)g.bits);
        return g.cellBase + ((spread3(x[0]) << 2) | (spread3(x[1]) << 1) | spread3(x[2]));
    }
    uint32_t x[2] = {ix, iy};
    hilbertTranspose<2>(x, (int)g.bits);
    return g.cellBase + ((spread2(x[0]) << 1) | spread2(x[1]));
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

// ---------------------------------------------------------------- radix sort
// Stable LSD radix sort of 32-bit keys carrying their input index. A pass
// handles one digit of at most 9 bits over tiles of kRadixTileKeys
// consecutive keys: a digit histogram per tile, stored digit-major so that
// one exclusive scan gives every tile its first output slot per digit, then a
// scatter that orders the tile by digit in shared memory and writes each
// digit's run out contiguously. Inside a tile each warp owns a contiguous
// quarter: per-warp digit counts, one exclusive scan over (digit, warp), then
// every key's slot is its warp's running slot for the digit plus its rank
// among the lanes of its round with the same digit (per-bit ballots). Equal
// keys keep their input order, so the output is the same on every run.
constexpr uint32_t kRadixTileKeys = 4096;
constexpr uint32_t kRadixHistBlock = 256;
constexpr uint32_t kRadixBlock = 128, kRadixWarps = kRadixBlock / 32, kRadixWarpKeys = kRadixTileKeys / kRadixWarps;
constexpr int kRadixMaxDigitBits = 9;
constexpr uint32_t kRadixMaxDigits = 1u << kRadixMaxDigitBits;

// lanes of the warp holding the same digit as this lane (0 for an invalid
// lane): one ballot per digit bit, the lanes agreeing on every bit
FCPWGB_D uint32_t digitPeers(uint32_t digit, int bits, bool valid) {
    uint32_t m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < kRadixMaxDigitBits; b++) {
        if (b < bits) {
            const bool set = (digit >> b) & 1u;
            const uint32_t v = __ballot_sync(0xffffffffu, set);
            m &= set ? v : ~v;
        }
    }
    return valid ? m : 0u;
}

__global__ void __launch_bounds__(kRadixHistBlock) kRadixHistogram(const uint32_t *__restrict__ keys, uint32_t n,
                                                                   int shift, int bits, uint32_t nTiles,
                                                                   uint32_t *hist) {
    const uint32_t mask = (1u << bits) - 1u;
    __shared__ uint32_t h[kRadixMaxDigits];
    for (uint32_t d = threadIdx.x; d <= mask; d += kRadixHistBlock) h[d] = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, base = blockIdx.x * kRadixTileKeys;
    for (uint32_t r = 0; r < kRadixTileKeys / kRadixHistBlock; r++) {
        const uint32_t i = base + r * kRadixHistBlock + threadIdx.x;
        const bool valid = i < n;
        const uint32_t digit = valid ? (__ldg(keys + i) >> shift) & mask : 0u;
        const uint32_t peers = digitPeers(digit, bits, valid);
        if (valid && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&h[digit], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d <= mask; d += kRadixHistBlock) hist[(size_t)d * nTiles + blockIdx.x] = h[d];
}

// valsIn null: the value of key i is i
__global__ void __launch_bounds__(kRadixBlock) kRadixScatter(const uint32_t *__restrict__ keysIn,
                                                             const uint32_t *__restrict__ valsIn, uint32_t n,
                                                             int shift, int bits, uint32_t nTiles,
                                                             const uint32_t *__restrict__ offsets, uint32_t *keysOut,
                                                             uint32_t *valsOut) {
    constexpr uint32_t kRounds = kRadixWarpKeys / 32;
    const uint32_t mask = (1u << bits) - 1u;
    __shared__ uint32_t sKeys[kRadixTileKeys], sVals[kRadixTileKeys];
    __shared__ uint32_t start[kRadixMaxDigits * kRadixWarps];  // (digit, warp): running slot in the tile
    __shared__ uint32_t tileStart[kRadixMaxDigits], globalStart[kRadixMaxDigits];
    __shared__ uint32_t warpSums[kRadixWarps];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, tile = blockIdx.x;
    const uint32_t base = tile * kRadixTileKeys, nd = mask + 1u, nEntries = nd * kRadixWarps;
    const uint32_t tileN = min(kRadixTileKeys, n - base);
    for (uint32_t k = threadIdx.x; k < nEntries; k += kRadixBlock) start[k] = 0;
    for (uint32_t d = threadIdx.x; d < nd; d += kRadixBlock) globalStart[d] = __ldg(offsets + (size_t)d * nTiles + tile);
    __syncthreads();
    // 1. digit counts of the warp's keys (read again in step 3, then from L1)
    const uint32_t wBase = base + warp * kRadixWarpKeys;
#pragma unroll 4
    for (uint32_t r = 0; r < kRounds; r++) {
        const uint32_t i = wBase + r * 32 + lane;
        const bool valid = i < n;
        const uint32_t digit = valid ? (__ldg(keysIn + i) >> shift) & mask : 0u;
        const uint32_t peers = digitPeers(digit, bits, valid);
        if (valid && (peers & ((1u << lane) - 1u)) == 0) start[digit * kRadixWarps + warp] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // 2. exclusive scan of start[] in (digit, warp) order
    const uint32_t per = (nEntries + kRadixBlock - 1) / kRadixBlock, e0 = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t k = 0; k < per; k++)
        if (e0 + k < nEntries) sum += start[e0 + k];
    uint32_t incl = sum;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
    }
    if (lane == 31) warpSums[warp] = incl;
    __syncthreads();
    uint32_t run = incl - sum;
    for (uint32_t w = 0; w < warp; w++) run += warpSums[w];
    for (uint32_t k = 0; k < per; k++) {
        if (e0 + k < nEntries) {
            uint32_t c = start[e0 + k];
            start[e0 + k] = run;
            run += c;
        }
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < nd; d += kRadixBlock) tileStart[d] = start[d * kRadixWarps];
    __syncthreads();
    // 3. stage the tile in digit order
#pragma unroll 4
    for (uint32_t r = 0; r < kRounds; r++) {
        const uint32_t i = wBase + r * 32 + lane;
        const bool valid = i < n;
        const uint32_t key = valid ? __ldg(keysIn + i) : 0u;
        const uint32_t digit = valid ? (key >> shift) & mask : 0u;
        const uint32_t peers = digitPeers(digit, bits, valid);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid) {
            const uint32_t slot = start[digit * kRadixWarps + warp] + rank;
            sKeys[slot] = key;
            sVals[slot] = valsIn ? __ldg(valsIn + i) : i;
        }
        __syncwarp();
        if (valid && rank == 0) start[digit * kRadixWarps + warp] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // 4. every digit's run of the tile goes out contiguously
    for (uint32_t s = threadIdx.x; s < tileN; s += kRadixBlock) {
        const uint32_t k = sKeys[s], d = (k >> shift) & mask;
        const uint32_t pos = globalStart[d] + s - tileStart[d];
        keysOut[pos] = k;
        valsOut[pos] = sVals[s];
    }
}

uint32_t radixTiles(uint32_t n) { return (n + kRadixTileKeys - 1) / kRadixTileKeys; }

size_t radixScratchWords(uint32_t n) {
    const uint32_t hist = kRadixMaxDigits * std::max(radixTiles(n), 1u);
    return (size_t)hist + batchScanTiles(hist) + 4;
}

cudaError_t radixSortIndices(uint32_t *keys0, uint32_t *keys1, uint32_t n, int keyBits, uint32_t *valsOut,
                             uint32_t *valsAlt, uint32_t *scratch, const uint32_t **sortedKeys, cudaStream_t s) {
    if (sortedKeys) *sortedKeys = keys0;
    if (n == 0) return cudaSuccess;
    keyBits = std::min(std::max(keyBits, 1), 32);
    const int passes = (keyBits + kRadixMaxDigitBits - 1) / kRadixMaxDigitBits;
    const int digitBits = (keyBits + passes - 1) / passes;
    const uint32_t mask = (1u << digitBits) - 1u, tiles = radixTiles(n), nHist = (mask + 1u) * tiles;
    uint32_t *hist = scratch, *tileSums = scratch + (size_t)kRadixMaxDigits * tiles;
    uint32_t *keys[2] = {keys0, keys1};
    const uint32_t *vin = nullptr;
    cudaError_t e;
    for (int p = 0; p < passes; p++) {
        const int shift = p * digitBits;
        uint32_t *vout = (passes - 1 - p) % 2 == 0 ? valsOut : valsAlt;  // the last pass writes valsOut
        kRadixHistogram<<<tiles, kRadixHistBlock, 0, s>>>(keys[p & 1], n, shift, digitBits, tiles, hist);
        if ((e = scanCounts(hist, nHist, tileSums, s)) != cudaSuccess) return e;
        kRadixScatter<<<tiles, kRadixBlock, 0, s>>>(keys[p & 1], vin, n, shift, digitBits, tiles, hist, keys[(p + 1) & 1],
                                                     vout);
        vin = vout;
    }
    if (sortedKeys) *sortedKeys = keys[passes & 1];
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
