// GPU BVH construction (a linear BVH): primitive centroids get Morton codes
// within their bounds, a stable radix sort orders them (equal codes keep
// primitive order), the binary radix tree over the sorted codes is built in
// parallel with one thread per inner node (Karras, "Maximizing parallelism
// in the construction of BVHs, octrees, and k-d trees", HPG 2012), subtrees
// of at most maxLeaf primitives become leaves, boxes and node counts are
// computed bottom-up with arrival counters, and every node finds its
// pre-order position by walking up to the root. The result is written in the
// interop layouts (32 B nodes in pre-order, left child = i + 1, primitives in
// leaf order), so every query kernel runs on it unchanged. Primitive boxes
// are the reference's: each vertex widened by FLT_EPSILON
// (bounding_volumes.h:38-49).
#include <algorithm>

#include "kernels.h"

namespace fcpwgb {

namespace {

constexpr uint32_t kNoNode = 0xffffffffu;
constexpr int kMaxWalk = 256;  // bound on any climb; trees deeper than 62 are rejected anyway

FCPWGB_D int orderedIntB(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
FCPWGB_D float orderedFloatB(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

FCPWGB_D float3 vtx(const float *pos, int dim, int32_t v) {
    return make_float3(pos[(size_t)v * dim], pos[(size_t)v * dim + 1], dim == 3 ? pos[(size_t)v * dim + 2] : 0.0f);
}

FCPWGB_D float3 centroid(const float *pos, const int32_t *idx, int dim, uint32_t p) {
    float3 c = make_float3(0.f, 0.f, 0.f);
    for (int j = 0; j < dim; j++) c = c + vtx(pos, dim, idx[(size_t)p * dim + j]);
    return c * (1.0f / (float)dim);
}

// bounds of the centroids (ordered-int atomics; cb initialised to +/- 3.4e38)
__global__ void kCentroidBounds(const float *pos, const int32_t *idx, int dim, uint32_t n, int *cb) {
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        float3 c = centroid(pos, idx, dim, p);
        float v[3] = {c.x, c.y, c.z};
        for (int a = 0; a < 3; a++) {
            lo[a] = fminf(lo[a], v[a]);
            hi[a] = fmaxf(hi[a], v[a]);
        }
    }
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    if ((threadIdx.x & 31u) == 0)
        for (int a = 0; a < 3; a++) {
            atomicMin(cb + a, orderedIntB(lo[a]));
            atomicMax(cb + 3 + a, orderedIntB(hi[a]));
        }
}

FCPWGB_D uint32_t spreadBits10(uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
FCPWGB_D uint32_t spreadBits16(uint32_t v) {  // 16 bits -> every second bit
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// flags any vertex index outside [0, nVertices) before a vertex is read
__global__ void kCheckIndices(const int32_t *idx, size_t nIdx, uint32_t nVertices, uint32_t *bad) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < nIdx; k += (size_t)gridDim.x * blockDim.x)
        if (idx[k] < 0 || (uint32_t)idx[k] >= nVertices) {
            atomicOr(bad, 1u);
            return;
        }
}

__global__ void kMortonCodes(const float *pos, const int32_t *idx, int dim, uint32_t n, const int *cb,
                             uint32_t *codes) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float3 c = centroid(pos, idx, dim, p);
    float v[3] = {c.x, c.y, c.z};
    const float cells = dim == 3 ? 1024.0f : 65536.0f;
    uint32_t q[3];
    for (int a = 0; a < 3; a++) {
        float lo = orderedFloatB(cb[a]), hi = orderedFloatB(cb[3 + a]);
        float t = (v[a] - lo) / fmaxf(hi - lo, 1e-30f) * cells;
        q[a] = (uint32_t)fminf(fmaxf(t, 0.0f), cells - 1.0f);
    }
    codes[p] = dim == 3 ? (spreadBits10(q[0]) | (spreadBits10(q[1]) << 1) | (spreadBits10(q[2]) << 2))
                        : (spreadBits16(q[0]) | (spreadBits16(q[1]) << 1));
}

// ---- Karras radix tree over sorted codes (ties broken by position)
FCPWGB_D int delta(const uint32_t *codes, uint32_t n, int i, int j) {
    if (j < 0 || j >= (int)n) return -1;
    uint32_t a = codes[i], b = codes[j];
    return a != b ? __clz(a ^ b) : 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// inner node i: children (inner id < n-1, or leaf n-1+k), range, parents
__global__ void kRadixTree(const uint32_t *codes, uint32_t n, uint32_t *left, uint32_t *right, uint32_t *first,
                           uint32_t *last, uint32_t *parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)n - 1) return;
    int d = delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1) >= 0 ? 1 : -1;
    int dMin = delta(codes, n, i, i - d);
    int lmax = 2;
    while (delta(codes, n, i, i + lmax * d) > dMin && lmax < (int)(2 * n)) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(codes, n, i, i + (l + t) * d) > dMin) l += t;
    int j = i + l * d;
    int dNode = delta(codes, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
        int t = (l + div - 1) / div;
        if (delta(codes, n, i, i + (s + t) * d) > dNode) s += t;
        if (t <= 1) break;
    }
    int g = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    uint32_t L = lo == g ? (n - 1 + (uint32_t)g) : (uint32_t)g;
    uint32_t R = hi == g + 1 ? (n - 1 + (uint32_t)g + 1) : (uint32_t)g + 1;
    left[i] = L;
    right[i] = R;
    first[i] = (uint32_t)lo;
    last[i] = (uint32_t)hi;
    parent[L] = (uint32_t)i;
    parent[R] = (uint32_t)i;
    if (i == 0) parent[0] = kNoNode;
}

FCPWGB_D uint32_t rangeFirst(uint32_t id, uint32_t n, const uint32_t *first) { return id >= n - 1 ? id - (n - 1) : first[id]; }
FCPWGB_D uint32_t rangeLast(uint32_t id, uint32_t n, const uint32_t *last) { return id >= n - 1 ? id - (n - 1) : last[id]; }

// final leaves: children of inner nodes of more than maxLeaf primitives that
// hold at most maxLeaf themselves
__global__ void kFinalLeaves(uint32_t n, uint32_t maxLeaf, const uint32_t *left, const uint32_t *right,
                             const uint32_t *first, const uint32_t *last, uint32_t *leafList, uint32_t *leafCount) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && n <= maxLeaf) {  // the root is the only leaf (node 0: inner, or the single primitive)
        leafList[atomicAdd(leafCount, 1u)] = 0;
        return;
    }
    if (i >= n - 1 || last[i] - first[i] + 1 <= maxLeaf) return;
    uint32_t ch[2] = {left[i], right[i]};
    for (int k = 0; k < 2; k++) {
        uint32_t c = ch[k];
        if (rangeLast(c, n, last) - rangeFirst(c, n, first) + 1 <= maxLeaf) leafList[atomicAdd(leafCount, 1u)] = c;
    }
}

// boxes and final-tree node counts, bottom-up from the final leaves
__global__ void kBuildBoxes(const float *pos, const int32_t *idx, const uint32_t *order, int dim, uint32_t n,
                            const uint32_t *leafList, const uint32_t *leafCount, const uint32_t *left,
                            const uint32_t *right, const uint32_t *first, const uint32_t *last,
                            const uint32_t *parent, float *boxes, uint32_t *sizes, uint32_t *arrivals,
                            uint32_t *errorWord) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= *leafCount) return;
    uint32_t node = leafList[t];
    const float eps = kFltEps;
    float lo[3] = {kFltMax, kFltMax, kFltMax}, hi[3] = {-kFltMax, -kFltMax, -kFltMax};
    for (uint32_t k = rangeFirst(node, n, first); k <= rangeLast(node, n, last); k++) {
        uint32_t p = order[k];
        for (int j = 0; j < dim; j++) {
            float3 v = vtx(pos, dim, idx[(size_t)p * dim + j]);
            float c[3] = {v.x, v.y, v.z};
            for (int a = 0; a < dim; a++) {
                lo[a] = fminf(lo[a], c[a] - eps);
                hi[a] = fmaxf(hi[a], c[a] + eps);
            }
        }
    }
    if (dim == 2) lo[2] = hi[2] = 0.0f;
    for (int a = 0; a < 3; a++) {
        boxes[(size_t)node * 6 + a] = lo[a];
        boxes[(size_t)node * 6 + 3 + a] = hi[a];
    }
    sizes[node] = 1;
    for (int step = 0; step < kMaxWalk; step++) {
        uint32_t p = parent[node];
        if (p == kNoNode) return;
        __threadfence();
        if (atomicAdd(arrivals + p, 1u) == 0) return;  // the sibling finishes the parent
        __threadfence();
        uint32_t L = left[p], R = right[p];
        for (int a = 0; a < 3; a++) {
            boxes[(size_t)p * 6 + a] = fminf(__ldcg(boxes + (size_t)L * 6 + a), __ldcg(boxes + (size_t)R * 6 + a));
            boxes[(size_t)p * 6 + 3 + a] =
                fmaxf(__ldcg(boxes + (size_t)L * 6 + 3 + a), __ldcg(boxes + (size_t)R * 6 + 3 + a));
        }
        sizes[p] = 1 + __ldcg(sizes + L) + __ldcg(sizes + R);
        node = p;
    }
    atomicOr(errorWord, kErrStepBudget);
}

// pre-order position of a final node: 0 for the root; a left child follows
// its parent, a right child follows its parent and the left sibling's subtree
FCPWGB_D bool preorderOf(uint32_t node, const uint32_t *parent, const uint32_t *left, const uint32_t *sizes,
                         uint32_t &pos, uint32_t &depth) {
    pos = 0;
    depth = 0;
    for (int step = 0; step < kMaxWalk; step++) {
        uint32_t p = parent[node];
        if (p == kNoNode) return true;
        pos += left[p] == node ? 1u : 1u + sizes[left[p]];
        depth++;
        node = p;
    }
    return false;
}

// writes one interop node record per final node
__global__ void kEmitNodes(uint32_t n, uint32_t maxLeaf, const uint32_t *leafList, const uint32_t *leafCount,
                           const uint32_t *left, const uint32_t *right, const uint32_t *first, const uint32_t *last,
                           const uint32_t *parent, const float *boxes, const uint32_t *sizes,
                           unsigned char *nodesOut, uint32_t *maxDepth, uint32_t *errorWord) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nLeaves = *leafCount, node;
    bool isLeaf;
    if (t < nLeaves) {
        node = leafList[t];
        isLeaf = true;
    } else {
        node = t - nLeaves;  // inner ids 0 .. n-2; only those above maxLeaf are final nodes
        if (node >= n - 1 || last[node] - first[node] + 1 <= maxLeaf) return;
        isLeaf = false;
    }
    uint32_t pos, depth;
    if (!preorderOf(node, parent, left, sizes, pos, depth)) {
        atomicOr(errorWord, kErrStepBudget);
        return;
    }
    atomicMax(maxDepth, depth);
    float *rec = reinterpret_cast<float *>(nodesOut + (size_t)pos * 32);
    for (int a = 0; a < 6; a++) rec[a] = boxes[(size_t)node * 6 + a];
    uint32_t *u = reinterpret_cast<uint32_t *>(rec + 6);
    if (isLeaf) {
        u[0] = rangeLast(node, n, last) - rangeFirst(node, n, first) + 1;
        u[1] = rangeFirst(node, n, first);
    } else {
        u[0] = 0;
        u[1] = 1 + sizes[left[node]];
    }
}

// primitives in leaf order: interop records (original index) and their vertices
__global__ void kEmitPrimitives(const float *pos, const int32_t *idx, const uint32_t *order, int dim, uint32_t n,
                                unsigned char *primsOut, int32_t *primVerts) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t p = order[k];
    float *rec = reinterpret_cast<float *>(primsOut + (size_t)k * (dim == 3 ? 40 : 28));
    for (int j = 0; j < dim; j++) {
        int32_t v = idx[(size_t)p * dim + j];
        primVerts[(size_t)k * dim + j] = v;
        float3 x = vtx(pos, dim, v);
        rec[3 * j] = x.x;
        rec[3 * j + 1] = x.y;
        rec[3 * j + 2] = dim == 3 ? x.z : 0.0f;
    }
    reinterpret_cast<uint32_t *>(rec)[3 * dim] = p;
}

}  // namespace

size_t lbvhScratchWords(uint32_t n) { return 27 * (size_t)n + radixScratchWords(n) + 16; }

cudaError_t launchCheckIndices(const int32_t *indices, size_t nIdx, uint32_t nVertices, uint32_t *bad, int numSMs,
                               cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess || nIdx == 0) return e;
    uint32_t blocks = (uint32_t)std::min<size_t>((nIdx + 255) / 256, (size_t)std::max(numSMs, 1) * 8u);
    kCheckIndices<<<blocks, 256, 0, s>>>(indices, nIdx, nVertices, bad);
    return cudaGetLastError();
}

// counters (device, 8 words): [0] final leaves, [1] deepest final node, [2..7] centroid bounds.
// Every vertex index must be in range (launchCheckIndices) before this runs.
cudaError_t launchBuildLbvh(const float *positions, const int32_t *indices, int dim, uint32_t n, uint32_t maxLeaf,
                            uint32_t *scratch, unsigned char *nodesOut, unsigned char *primsOut,
                            int32_t *primVertsOut, uint32_t *counters, uint32_t *errorWord, int numSMs,
                            cudaStream_t s) {
    if (n == 0 || maxLeaf == 0 || n >= (1u << 30)) return cudaErrorInvalidValue;
    const size_t nodes = 2 * (size_t)n;
    uint32_t *p = scratch;
    uint32_t *codes0 = p; p += n;
    uint32_t *codes1 = p; p += n;
    uint32_t *ids = p; p += n;
    uint32_t *idsAlt = p; p += n;
    uint32_t *left = p; p += n;
    uint32_t *right = p; p += n;
    uint32_t *first = p; p += n;
    uint32_t *last = p; p += n;
    uint32_t *parent = p; p += nodes;
    uint32_t *sizes = p; p += nodes;
    uint32_t *arrivals = p; p += nodes;
    uint32_t *leafList = p; p += n;
    float *boxes = reinterpret_cast<float *>(p); p += nodes * 6;
    uint32_t *radix = p;
    int *cb = reinterpret_cast<int *>(counters + 2);

    cudaError_t e;
    if ((e = cudaMemsetAsync(counters, 0, 2 * sizeof(uint32_t), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(cb, 0x7f, 3 * sizeof(int), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(cb + 3, 0x80, 3 * sizeof(int), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(arrivals, 0, nodes * sizeof(uint32_t), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(parent, 0xff, nodes * sizeof(uint32_t), s)) != cudaSuccess) return e;
    const uint32_t blocks = (n + 255) / 256;
    kCentroidBounds<<<std::min<uint32_t>(blocks, (uint32_t)std::max(numSMs, 1) * 8u), 256, 0, s>>>(
        positions, indices, dim, n, cb);
    kMortonCodes<<<blocks, 256, 0, s>>>(positions, indices, dim, n, cb, codes0);
    const uint32_t *codes = codes0;
    if ((e = radixSortIndices(codes0, codes1, n, dim == 3 ? 30 : 32, ids, idsAlt, radix, &codes, s)) != cudaSuccess)
        return e;
    if (n > 1) kRadixTree<<<(n - 1 + 255) / 256, 256, 0, s>>>(codes, n, left, right, first, last, parent);
    kFinalLeaves<<<(std::max(n - 1, 1u) + 255) / 256, 256, 0, s>>>(n, maxLeaf, left, right, first, last, leafList,
                                                                  counters);
    kBuildBoxes<<<blocks, 256, 0, s>>>(positions, indices, ids, dim, n, leafList, counters, left, right, first, last,
                                       parent, boxes, sizes, arrivals, errorWord);
    kEmitNodes<<<(2 * n + 255) / 256, 256, 0, s>>>(n, maxLeaf, leafList, counters, left, right, first, last, parent,
                                                    boxes, sizes, nodesOut, counters + 1, errorWord);
    kEmitPrimitives<<<blocks, 256, 0, s>>>(positions, indices, ids, dim, n, primsOut, primVertsOut);
    return cudaGetLastError();
}

}  // namespace fcpwgb
