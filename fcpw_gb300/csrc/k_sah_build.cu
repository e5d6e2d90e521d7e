// The reference's binned-SAH BVH (bvh.inl:1-234, Scene::build with
// vectorize=false: 8 buckets, leaf <= 4, depth cut at 62) built on the
// device, node for node the tree the host builder (host_bvh.cpp) and the
// reference make.
//
// Large nodes (more than kSmall references) are split level by level with
// the whole GPU: per node the box of the references and the padded box of
// their centroids, the 8 bucket boxes and counts per axis (blocks of
// kChunk references reduce in shared memory; min/max through order-preserving
// integer atomics, so the result does not depend on the order), then one
// thread per node runs the bucket sweep in the host's operation order and
// picks the split. The partition reproduces the reference's in-place
// partition (bvh.inl:114-140) exactly: references below the split keep their
// order (prefix sums), and the others end in the order that partition's
// swaps leave them, which has a closed form: the element ending at position
// r of the node (r at or after the split count P) is found by following
// u -> P(u) from u = r while the element at u is below the split, P(u) being
// the number of elements below the split before u; the chains are resolved
// by pointer jumping. Subtrees of at most kSmall references are then built by
// one thread each, with the host's recursion and arithmetic. The arithmetic
// is written with explicit round-to-nearest operations (no fused
// multiply-adds), as the host build is compiled without contraction.
#include <algorithm>
#include <cstring>
#include <functional>
#include <vector>

#include "kernels.h"
#include "scene.h"

namespace fcpwgb {

namespace {

constexpr int kNB = 8;                // buckets (bvh.h:77 default)
constexpr int kLeafRefs = 4;          // leaf size (fcpw.inl:813)
constexpr uint32_t kCutDepth = 62;    // FCPW_BVH_MAX_DEPTH - 2 (bvh.inl:170)
constexpr uint32_t kSmall = 64;       // subtrees of at most this many references: one thread each
constexpr uint32_t kChunk = 2048;     // references per block in the level passes
constexpr uint32_t kLB = 256;         // threads per block in the level passes
constexpr int kSeqStack = 130;

enum { kLongestAxis = 0, kSurfaceArea = 1, kOverlapSurfaceArea = 2, kVolume = 3, kOverlapVolume = 4 };

FCPWGB_D float hmin(float x, float y) { return y < x ? y : x; }  // cwiseMin of the host build
FCPWGB_D float hmax(float x, float y) { return x < y ? y : x; }
FCPWGB_HD int ordInt(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
FCPWGB_D float ordFloat(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

template<int D> struct HBox {
    float lo[D], hi[D];
    FCPWGB_D void clear() {
        for (int a = 0; a < D; a++) { lo[a] = kFltMax; hi[a] = -kFltMax; }
    }
    FCPWGB_D void addBox(const HBox &b) {
        for (int a = 0; a < D; a++) { lo[a] = hmin(lo[a], b.lo[a]); hi[a] = hmax(hi[a], b.hi[a]); }
    }
    FCPWGB_D void addPoint(const float *p) {  // Box::expand(Vec): the point widened by FLT_EPSILON
        for (int a = 0; a < D; a++) {
            lo[a] = hmin(lo[a], __fsub_rn(p[a], kFltEps));
            hi[a] = hmax(hi[a], __fadd_rn(p[a], kFltEps));
        }
    }
    FCPWGB_D float ext(int a) const { return __fsub_rn(hi[a], lo[a]); }
    FCPWGB_D float surfaceArea() const {
        float e[D];
        for (int a = 0; a < D; a++) e[a] = hmax(ext(a), 1e-5f);
        if (D == 3) {
            float p = __fmul_rn(e[0], __fmul_rn(e[1], e[2]));
            float q0 = __fdiv_rn(p, e[0]), q1 = __fdiv_rn(p, e[1]), q2 = __fdiv_rn(p, e[2 % D]);
            return __fmul_rn(2.0f, __fadd_rn(q0, __fadd_rn(q1, q2)));
        }
        float p = __fmul_rn(e[0], e[1]);
        return __fmul_rn(2.0f, __fadd_rn(__fdiv_rn(p, e[0]), __fdiv_rn(p, e[1])));
    }
    FCPWGB_D float volume() const {
        if (D == 3) return __fmul_rn(ext(0), __fmul_rn(ext(1), ext(2 % D)));
        return __fmul_rn(ext(0), ext(1));
    }
    FCPWGB_D HBox meet(const HBox &b) const {
        HBox r;
        for (int a = 0; a < D; a++) { r.lo[a] = hmax(lo[a], b.lo[a]); r.hi[a] = hmin(hi[a], b.hi[a]); }
        return r;
    }
    FCPWGB_D bool valid() const {
        for (int a = 0; a < D; a++)
            if (!(hi[a] >= lo[a])) return false;
        return true;
    }
    FCPWGB_D int maxDim() const {
        int idx = 0;
        float best = ext(0);
        for (int a = 1; a < D; a++)
            if (ext(a) > best) { best = ext(a); idx = a; }
        return idx;
    }
};

template<int D> FCPWGB_D HBox<D> loadBox(const float *box, uint32_t r) {
    HBox<D> b;
    for (int a = 0; a < D; a++) { b.lo[a] = box[(size_t)r * 6 + a]; b.hi[a] = box[(size_t)r * 6 + 3 + a]; }
    return b;
}

// computeSplitCost, bvh.inl:4-37 (packLeaves off)
template<int D> FCPWGB_D float splitCost(int heur, const HBox<D> &l, const HBox<D> &r, int nl, int nr) {
    float cost = kFltMax;
    if (heur == kSurfaceArea) {
        cost = __fadd_rn(__fmul_rn((float)nl, l.surfaceArea()), __fmul_rn((float)nr, r.surfaceArea()));
    } else if (heur == kOverlapSurfaceArea) {
        HBox<D> bi = l.meet(r);
        cost = __fmul_rn(__fadd_rn(__fdiv_rn((float)nl, r.surfaceArea()), __fdiv_rn((float)nr, l.surfaceArea())),
                         fabsf(bi.surfaceArea()));
        if (!bi.valid()) cost = -cost;
    } else if (heur == kVolume) {
        cost = __fadd_rn(__fmul_rn((float)nl, l.volume()), __fmul_rn((float)nr, r.volume()));
    } else if (heur == kOverlapVolume) {
        HBox<D> bi = l.meet(r);
        cost = __fmul_rn(__fadd_rn(__fdiv_rn((float)nl, r.volume()), __fdiv_rn((float)nr, l.volume())),
                         fabsf(bi.volume()));
        if (!bi.valid()) cost = -cost;
    }
    return cost;
}

template<int D> FCPWGB_D int bucketOf(float c, float lo, float width) {
    int b = __float2int_rz(__fdiv_rn(__fsub_rn(c, lo), width));
    return b < 0 ? 0 : (b > kNB - 1 ? kNB - 1 : b);
}

// the bucket sweep of computeObjectSplit (bvh.inl:40-111) over given buckets of one axis
template<int D>
FCPWGB_D void sweepAxis(int heur, int dim, const HBox<D> &bb, float width, const HBox<D> (&bucket)[kNB],
                        const int (&count)[kNB], float &best, int &bestDim, float &bestCoord) {
    HBox<D> right[kNB];
    int rightCount[kNB];
    HBox<D> acc;
    acc.clear();
    for (int b = kNB - 1; b > 0; b--) {
        acc.addBox(bucket[b]);
        right[b] = acc;
        rightCount[b] = count[b] + (b != kNB - 1 ? rightCount[b + 1] : 0);
    }
    HBox<D> left;
    left.clear();
    int nLeft = 0;
    for (int b = 1; b < kNB; b++) {
        left.addBox(bucket[b - 1]);
        nLeft += count[b - 1];
        if (nLeft > 0 && rightCount[b] > 0) {
            float cost = splitCost<D>(heur, left, right[b], nLeft, rightCount[b]);
            if (cost < best) {
                best = cost;
                bestDim = dim;
                bestCoord = __fadd_rn(bb.lo[dim], __fmul_rn((float)b, width));
            }
        }
    }
}

// ------------------------------------------------------------ one thread per subtree
struct SeqEntry {
    uint32_t start, end, depth;
    int parent;
};

// HostBvh::buildRecursive for one subtree, in place on its references;
// nodes in pre-order at out[0..), leaf offsets absolute, inner offsets relative
template<int D>
__global__ void kSeqSubtrees(int heur, const uint32_t *__restrict__ subStart, const uint32_t *__restrict__ subEnd,
                             const uint32_t *__restrict__ subDepth, const uint32_t *__restrict__ subBuf,
                             const uint32_t *__restrict__ subBase, uint32_t nSub, float *box0, float *cent0,
                             uint32_t *id0, float *box1, float *cent1, uint32_t *id1, unsigned char *nodesOut,
                             uint32_t *subCount, uint32_t *errorWord) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nSub) return;
    float *box = subBuf[i] ? box1 : box0;
    float *cent = subBuf[i] ? cent1 : cent0;
    uint32_t *id = subBuf[i] ? id1 : id0;
    float *outF = reinterpret_cast<float *>(nodesOut + (size_t)subBase[i] * 32);
    uint32_t *outU = reinterpret_cast<uint32_t *>(outF);
    SeqEntry stack[kSeqStack];
    int sp = 0;
    stack[0] = {subStart[i], subEnd[i], subDepth[i], -1};
    uint32_t count = 0;
    while (sp >= 0) {
        SeqEntry e = stack[sp--];
        const uint32_t me = count++;
        const uint32_t n = e.end - e.start;
        HBox<D> bb, bc;
        bb.clear();
        bc.clear();
        for (uint32_t p = e.start; p < e.end; p++) {
            bb.addBox(loadBox<D>(box, p));
            bc.addPoint(cent + (size_t)p * 3);
        }
        for (int a = 0; a < 3; a++) {
            outF[(size_t)me * 8 + a] = a < D ? bb.lo[a] : 0.0f;
            outF[(size_t)me * 8 + 3 + a] = a < D ? bb.hi[a] : 0.0f;
        }
        const bool leaf = n <= (uint32_t)kLeafRefs || e.depth == kCutDepth;
        outU[(size_t)me * 8 + 6] = leaf ? n : 0u;
        outU[(size_t)me * 8 + 7] = leaf ? e.start : 0u;
        if (e.parent >= 0 && me != (uint32_t)e.parent + 1) outU[(size_t)e.parent * 8 + 7] = me - (uint32_t)e.parent;
        if (leaf) continue;
        // split (computeObjectSplit)
        float best = kFltMax, coord = 0.0f;
        int dimSel = -1;
        if (heur != kLongestAxis) {
            for (int dim = 0; dim < D; dim++) {
                float extent = bb.ext(dim);
                if (extent < 1e-6f) continue;
                float width = __fdiv_rn(extent, (float)kNB);
                HBox<D> bucket[kNB];
                int cnt[kNB];
                for (int b = 0; b < kNB; b++) { bucket[b].clear(); cnt[b] = 0; }
                for (uint32_t p = e.start; p < e.end; p++) {
                    int b = bucketOf<D>(cent[(size_t)p * 3 + dim], bb.lo[dim], width);
                    bucket[b].addBox(loadBox<D>(box, p));
                    cnt[b] += 1;
                }
                sweepAxis<D>(heur, dim, bb, width, bucket, cnt, best, dimSel, coord);
            }
        }
        if (dimSel == -1) {
            dimSel = bc.maxDim();
            coord = __fmul_rn(__fadd_rn(bc.lo[dimSel], bc.hi[dimSel]), 0.5f);
        }
        // in-place partition (performObjectSplit)
        uint32_t mid = e.start;
        for (uint32_t p = e.start; p < e.end; p++) {
            if (cent[(size_t)p * 3 + dimSel] < coord) {
                if (p != mid) {
                    for (int k = 0; k < 6; k++) {
                        float t = box[(size_t)p * 6 + k];
                        box[(size_t)p * 6 + k] = box[(size_t)mid * 6 + k];
                        box[(size_t)mid * 6 + k] = t;
                    }
                    for (int k = 0; k < 3; k++) {
                        float t = cent[(size_t)p * 3 + k];
                        cent[(size_t)p * 3 + k] = cent[(size_t)mid * 3 + k];
                        cent[(size_t)mid * 3 + k] = t;
                    }
                    uint32_t t = id[p];
                    id[p] = id[mid];
                    id[mid] = t;
                }
                mid++;
            }
        }
        if (mid == e.start || mid == e.end) mid = e.start + n / 2;
        if (sp + 2 >= kSeqStack) {
            atomicOr(errorWord, kErrStackOverflow);
            break;
        }
        stack[++sp] = {mid, e.end, e.depth + 1, (int)me};
        stack[++sp] = {e.start, mid, e.depth + 1, (int)me};
    }
    subCount[i] = count;
}

// ------------------------------------------------------------ level passes (large nodes)
// per node: 12 ordered ints (box lo/hi, centroid box lo/hi, 3 each), bins:
// 3 axes x 8 buckets x 7 (lo 3, hi 3 ordered ints, count)
constexpr int kBinInts = 3 * kNB * 7;

template<int D>
__global__ void kRefInit(const float *__restrict__ pos, const int32_t *__restrict__ idx, uint32_t n, float *box,
                         float *cent, uint32_t *id) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float v[3][3];
    for (int j = 0; j < D; j++) {
        int32_t k = idx[(size_t)p * D + j];
        for (int a = 0; a < D; a++) v[j][a] = pos[(size_t)k * D + a];
    }
    HBox<D> b;
    for (int a = 0; a < D; a++) {  // Box::fromPoint(pa), then expand(pb) [, expand(pc)]
        b.lo[a] = __fsub_rn(v[0][a], kFltEps);
        b.hi[a] = __fadd_rn(v[0][a], kFltEps);
    }
    for (int j = 1; j < D; j++) b.addPoint(v[j]);
    for (int a = 0; a < 3; a++) {
        box[(size_t)p * 6 + a] = a < D ? b.lo[a] : 0.0f;
        box[(size_t)p * 6 + 3 + a] = a < D ? b.hi[a] : 0.0f;
        float c = 0.0f;
        if (a < D)
            c = D == 3 ? __fdiv_rn(__fadd_rn(__fadd_rn(v[0][a], v[1][a]), v[2 % D][a]), 3.0f)
                       : __fmul_rn(__fadd_rn(v[0][a], v[1][a]), 0.5f);
        cent[(size_t)p * 3 + a] = c;
    }
    id[p] = p;
}

__global__ void kInitLevel(uint32_t nNodes, int *bounds, int *bins, uint32_t *counts) {
    uint32_t j = blockIdx.x;
    if (j >= nNodes) return;
    const int hiInit = ordInt(-kFltMax), loInit = ordInt(kFltMax);
    for (int k = threadIdx.x; k < 12; k += blockDim.x) bounds[j * 12 + k] = (k % 6) < 3 ? loInit : hiInit;
    for (int k = threadIdx.x; k < kBinInts; k += blockDim.x) {
        int f = k % 7;
        bins[j * kBinInts + k] = f == 6 ? 0 : (f < 3 ? loInit : hiInit);
    }
    (void)counts;
}

struct LevelMap {
    const uint32_t *blkNode, *blkBegin, *nodeStart, *nodeEnd;
};

template<int D>
__global__ void __launch_bounds__(kLB) kLevelBounds(LevelMap m, const float *__restrict__ box,
                                                    const float *__restrict__ cent, int *bounds) {
    __shared__ int s[12];
    const uint32_t j = m.blkNode[blockIdx.x], b0 = m.blkBegin[blockIdx.x];
    const uint32_t b1 = min(b0 + kChunk, m.nodeEnd[j]);
    if (threadIdx.x < 12) s[threadIdx.x] = (threadIdx.x % 6) < 3 ? ordInt(kFltMax) : ordInt(-kFltMax);
    __syncthreads();
    HBox<D> bb, bc;
    bb.clear();
    bc.clear();
    for (uint32_t p = b0 + threadIdx.x; p < b1; p += kLB) {
        bb.addBox(loadBox<D>(box, p));
        bc.addPoint(cent + (size_t)p * 3);
    }
    for (int a = 0; a < D; a++) {
        atomicMin(&s[a], ordInt(bb.lo[a]));
        atomicMax(&s[3 + a], ordInt(bb.hi[a]));
        atomicMin(&s[6 + a], ordInt(bc.lo[a]));
        atomicMax(&s[9 + a], ordInt(bc.hi[a]));
    }
    __syncthreads();
    if (threadIdx.x < 12 && (threadIdx.x % 3) < D) {
        int k = threadIdx.x;
        if ((k % 6) < 3) atomicMin(&bounds[j * 12 + k], s[k]);
        else atomicMax(&bounds[j * 12 + k], s[k]);
    }
}

template<int D> FCPWGB_D void decodeBounds(const int *b, HBox<D> &bb, HBox<D> &bc) {
    for (int a = 0; a < D; a++) {
        bb.lo[a] = ordFloat(b[a]);
        bb.hi[a] = ordFloat(b[3 + a]);
        bc.lo[a] = ordFloat(b[6 + a]);
        bc.hi[a] = ordFloat(b[9 + a]);
    }
}

template<int D>
__global__ void __launch_bounds__(kLB) kLevelBins(LevelMap m, int heur, const float *__restrict__ box,
                                                  const float *__restrict__ cent, const int *__restrict__ bounds,
                                                  int *bins) {
    __shared__ int s[kBinInts];
    const uint32_t j = m.blkNode[blockIdx.x], b0 = m.blkBegin[blockIdx.x];
    const uint32_t b1 = min(b0 + kChunk, m.nodeEnd[j]);
    for (int k = threadIdx.x; k < kBinInts; k += kLB) {
        int f = k % 7;
        s[k] = f == 6 ? 0 : (f < 3 ? ordInt(kFltMax) : ordInt(-kFltMax));
    }
    __syncthreads();
    if (heur != kLongestAxis) {
        HBox<D> bb, bc;
        decodeBounds<D>(bounds + j * 12, bb, bc);
        for (uint32_t p = b0 + threadIdx.x; p < b1; p += kLB) {
            HBox<D> rb = loadBox<D>(box, p);
            for (int dim = 0; dim < D; dim++) {
                float extent = bb.ext(dim);
                if (extent < 1e-6f) continue;
                float width = __fdiv_rn(extent, (float)kNB);
                int b = bucketOf<D>(cent[(size_t)p * 3 + dim], bb.lo[dim], width);
                int *q = s + (dim * kNB + b) * 7;
                for (int a = 0; a < D; a++) {
                    atomicMin(q + a, ordInt(rb.lo[a]));
                    atomicMax(q + 3 + a, ordInt(rb.hi[a]));
                }
                atomicAdd(q + 6, 1);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kBinInts; k += kLB) {
        int f = k % 7;
        if (f == 6) {
            if (s[k]) atomicAdd(&bins[j * kBinInts + k], s[k]);
        } else if ((f % 3) < D) {
            if (f < 3) atomicMin(&bins[j * kBinInts + k], s[k]);
            else atomicMax(&bins[j * kBinInts + k], s[k]);
        }
    }
}

// split[j] = (axis, coordinate bits)
template<int D>
__global__ void kLevelSplit(uint32_t nNodes, int heur, const int *__restrict__ bounds, const int *__restrict__ bins,
                            uint32_t *split) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nNodes) return;
    HBox<D> bb, bc;
    decodeBounds<D>(bounds + j * 12, bb, bc);
    float best = kFltMax, coord = 0.0f;
    int dimSel = -1;
    if (heur != kLongestAxis) {
        for (int dim = 0; dim < D; dim++) {
            float extent = bb.ext(dim);
            if (extent < 1e-6f) continue;
            float width = __fdiv_rn(extent, (float)kNB);
            HBox<D> bucket[kNB];
            int cnt[kNB];
            for (int b = 0; b < kNB; b++) {
                const int *q = bins + j * kBinInts + (dim * kNB + b) * 7;
                for (int a = 0; a < D; a++) {
                    bucket[b].lo[a] = ordFloat(q[a]);
                    bucket[b].hi[a] = ordFloat(q[3 + a]);
                }
                cnt[b] = q[6];
            }
            sweepAxis<D>(heur, dim, bb, width, bucket, cnt, best, dimSel, coord);
        }
    }
    if (dimSel == -1) {
        dimSel = bc.maxDim();
        coord = __fmul_rn(__fadd_rn(bc.lo[dimSel], bc.hi[dimSel]), 0.5f);
    }
    split[2 * j] = (uint32_t)dimSel;
    split[2 * j + 1] = __float_as_uint(coord);
}

// references below the split per block
__global__ void __launch_bounds__(kLB) kLevelCount(LevelMap m, const float *__restrict__ cent,
                                                   const uint32_t *__restrict__ split, uint32_t *blkCount) {
    __shared__ uint32_t s;
    const uint32_t j = m.blkNode[blockIdx.x], b0 = m.blkBegin[blockIdx.x];
    const uint32_t b1 = min(b0 + kChunk, m.nodeEnd[j]);
    const uint32_t dim = split[2 * j];
    const float coord = __uint_as_float(split[2 * j + 1]);
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    uint32_t c = 0;
    for (uint32_t p = b0 + threadIdx.x; p < b1; p += kLB) c += cent[(size_t)p * 3 + dim] < coord ? 1u : 0u;
    atomicAdd(&s, c);
    __syncthreads();
    if (threadIdx.x == 0) blkCount[blockIdx.x] = s;
}

// per node: exclusive scan of its blocks' counts (blocks of a node are consecutive)
__global__ void kLevelScan(uint32_t nNodes, const uint32_t *__restrict__ nodeBlk0, const uint32_t *__restrict__ nodeBlkN,
                           const uint32_t *__restrict__ blkCount, uint32_t *blkBase, uint32_t *below) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nNodes) return;
    uint32_t run = 0;
    for (uint32_t b = nodeBlk0[j]; b < nodeBlk0[j] + nodeBlkN[j]; b++) {
        blkBase[b] = run;
        run += blkCount[b];
    }
    below[j] = run;
}

// P(u) (position among the node's below-split references) and the first jump
// J(u) = start + P(u) for those below the split, u otherwise
__global__ void __launch_bounds__(kLB) kLevelRank(LevelMap m, const float *__restrict__ cent,
                                                  const uint32_t *__restrict__ split,
                                                  const uint32_t *__restrict__ blkBase, uint32_t *rank, uint32_t *jump) {
    __shared__ uint32_t warpSum[kLB / 32];
    __shared__ uint32_t run;
    const uint32_t j = m.blkNode[blockIdx.x], b0 = m.blkBegin[blockIdx.x];
    const uint32_t start = m.nodeStart[j], b1 = min(b0 + kChunk, m.nodeEnd[j]);
    const uint32_t dim = split[2 * j];
    const float coord = __uint_as_float(split[2 * j + 1]);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) run = blkBase[blockIdx.x];
    __syncthreads();
    for (uint32_t r = 0; r < kChunk / kLB; r++) {
        const uint32_t p = b0 + r * kLB + threadIdx.x;
        const bool valid = p < b1;
        const bool below = valid && cent[(size_t)p * 3 + dim] < coord;
        const uint32_t ball = __ballot_sync(0xffffffffu, below);
        if (lane == 0) warpSum[warp] = __popc(ball);
        __syncthreads();
        uint32_t before = run;
        for (uint32_t w = 0; w < warp; w++) before += warpSum[w];
        before += __popc(ball & ((1u << lane) - 1u));
        if (valid) {
            rank[p] = below ? before : 0xffffffffu;
            jump[p] = below ? start + before : p;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (uint32_t w = 0; w < kLB / 32; w++) t += warpSum[w];
            run += t;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kLB) kLevelJump(LevelMap m, const uint32_t *__restrict__ jin, uint32_t *jout) {
    const uint32_t j = m.blkNode[blockIdx.x], b0 = m.blkBegin[blockIdx.x];
    const uint32_t b1 = min(b0 + kChunk, m.nodeEnd[j]);
    for (uint32_t p = b0 + threadIdx.x; p < b1; p += kLB) jout[p] = jin[jin[p]];
}

FCPWGB_D void copyRef(const float *bs, const float *cs, const uint32_t *is, uint32_t from, float *bd, float *cd,
                      uint32_t *id, uint32_t to) {
    for (int k = 0; k < 6; k++) bd[(size_t)to * 6 + k] = bs[(size_t)from * 6 + k];
    for (int k = 0; k < 3; k++) cd[(size_t)to * 3 + k] = cs[(size_t)from * 3 + k];
    id[to] = is[from];
}

// the node's references in the order the in-place partition leaves them
__global__ void __launch_bounds__(kLB) kLevelGather(LevelMap m, const uint32_t *__restrict__ below,
                                                    const uint32_t *__restrict__ rank, const uint32_t *__restrict__ jump,
                                                    const float *bs, const float *cs, const uint32_t *is, float *bd,
                                                    float *cd, uint32_t *id) {
    const uint32_t j = m.blkNode[blockIdx.x], b0 = m.blkBegin[blockIdx.x];
    const uint32_t start = m.nodeStart[j], end = m.nodeEnd[j], b1 = min(b0 + kChunk, end);
    const uint32_t P = below[j], n = end - start;
    const bool fallback = P == 0 || P == n;  // every swap a no-op: the order stays
    for (uint32_t p = b0 + threadIdx.x; p < b1; p += kLB) {
        if (fallback) {
            copyRef(bs, cs, is, p, bd, cd, id, p);
            continue;
        }
        if (rank[p] != 0xffffffffu) copyRef(bs, cs, is, p, bd, cd, id, start + rank[p]);
        if (p - start >= P) copyRef(bs, cs, is, jump[p], bd, cd, id, p);
    }
}

__global__ void kFinalOrder(const uint32_t *__restrict__ subStart, const uint32_t *__restrict__ subEnd,
                            const uint32_t *__restrict__ subBuf, uint32_t nSub, const uint32_t *id0,
                            const uint32_t *id1, uint32_t *order) {
    uint32_t i = blockIdx.x;
    if (i >= nSub) return;
    const uint32_t *src = subBuf[i] ? id1 : id0;
    for (uint32_t p = subStart[i] + threadIdx.x; p < subEnd[i]; p += blockDim.x) order[p] = src[p];
}

__global__ void kPlaceSubtrees(const uint32_t *__restrict__ subBase, const uint32_t *__restrict__ subCount,
                               const uint32_t *__restrict__ subPos, uint32_t nSub, const uint4 *scratchNodes,
                               uint4 *nodes) {
    uint32_t i = blockIdx.x;
    if (i >= nSub) return;
    for (uint32_t k = threadIdx.x; k < subCount[i]; k += blockDim.x) {
        nodes[2 * ((size_t)subPos[i] + k)] = scratchNodes[2 * ((size_t)subBase[i] + k)];
        nodes[2 * ((size_t)subPos[i] + k) + 1] = scratchNodes[2 * ((size_t)subBase[i] + k) + 1];
    }
}

__global__ void kPlaceNodes(const unsigned char *recs, const uint32_t *pos, uint32_t n, unsigned char *nodes) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    for (int b = 0; b < 32; b++) nodes[(size_t)pos[k] * 32 + b] = recs[(size_t)k * 32 + b];
}

__global__ void kEmitSahPrimitives(const float *pos, const int32_t *idx, const uint32_t *order, int dim, uint32_t n,
                                   unsigned char *primsOut, int32_t *primVerts) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t p = order[k];
    float *rec = reinterpret_cast<float *>(primsOut + (size_t)k * (dim == 3 ? 40 : 28));
    for (int j = 0; j < dim; j++) {
        int32_t v = idx[(size_t)p * dim + j];
        primVerts[(size_t)k * dim + j] = v;
        for (int a = 0; a < 3; a++) rec[3 * j + a] = a < dim ? pos[(size_t)v * dim + a] : 0.0f;
    }
    reinterpret_cast<uint32_t *>(rec)[3 * dim] = p;
}

template<class T> int uploadVec(DeviceBuffer &b, const std::vector<T> &v, cudaStream_t st) {
    return b.upload(v.data(), v.size() * sizeof(T), st);
}

struct TopNode {       // a large node of the host-side level tree
    int left = -1, right = -1, sub = -1;
    int bounds[12];
};

}  // namespace

// Builds the reference SAH tree of positions/indices (device arrays, indices
// checked by the caller) on stream st. nodesOut: nNodes interop nodes,
// primsOut: n interop primitives, vertsOut: n * dim vertex indices.
int buildSahTree(int dim, int heuristic, const float *positions, const int32_t *indices, uint32_t n,
                 uint32_t *errorWord, cudaStream_t st, DeviceBuffer &nodesOut, DeviceBuffer &primsOut,
                 DeviceBuffer &vertsOut, uint32_t &nNodes) {
    int rc;
    cudaError_t e;
    DeviceBuffer box[2], cent[2], ids[2];
    for (int b = 0; b < 2; b++) {
        if ((rc = box[b].ensure((size_t)n * 24)) || (rc = cent[b].ensure((size_t)n * 12)) ||
            (rc = ids[b].ensure((size_t)n * 4)))
            return rc;
    }
    const uint32_t g = (n + 255) / 256;
    if (dim == 3)
        kRefInit<3><<<g, 256, 0, st>>>(positions, indices, n, (float *)box[0].ptr, (float *)cent[0].ptr,
                                       (uint32_t *)ids[0].ptr);
    else
        kRefInit<2><<<g, 256, 0, st>>>(positions, indices, n, (float *)box[0].ptr, (float *)cent[0].ptr,
                                       (uint32_t *)ids[0].ptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "reference boxes");

    struct Pending { uint32_t start, end, depth; int top; bool right; };
    std::vector<TopNode> tops;
    std::vector<uint32_t> sStart, sEnd, sDepth, sBuf;
    std::vector<std::pair<int, bool>> sParent;  // (top node, is right child) of every subtree, -1 for the root
    std::vector<Pending> level;
    auto addChild = [&](uint32_t s0, uint32_t s1, uint32_t depth, int parent, bool right, int buf,
                        std::vector<Pending> &next) {
        if (s1 - s0 <= kSmall || depth >= kCutDepth) {
            int k = (int)sStart.size();
            sStart.push_back(s0);
            sEnd.push_back(s1);
            sDepth.push_back(depth);
            sBuf.push_back((uint32_t)buf);
            sParent.push_back({parent, right});
            if (parent >= 0) (right ? tops[parent].right : tops[parent].left) = -2 - k;
        } else {
            next.push_back({s0, s1, depth, parent, right});
        }
    };
    addChild(0, n, 0, -1, false, 0, level);
    int buf = 0;
    DeviceBuffer mapBuf, nodeBuf, boundsBuf, binsBuf, splitBuf, cntBuf, baseBuf, belowBuf, rankBuf, jumpBuf[2];
    while (!level.empty()) {
        const uint32_t nn = (uint32_t)level.size();
        std::vector<uint32_t> blkNode, blkBegin, nodeStart(nn), nodeEnd(nn), nodeBlk0(nn), nodeBlkN(nn);
        uint32_t maxLen = 0;
        for (uint32_t j = 0; j < nn; j++) {
            nodeStart[j] = level[j].start;
            nodeEnd[j] = level[j].end;
            nodeBlk0[j] = (uint32_t)blkNode.size();
            for (uint32_t b = level[j].start; b < level[j].end; b += kChunk) {
                blkNode.push_back(j);
                blkBegin.push_back(b);
            }
            nodeBlkN[j] = (uint32_t)blkNode.size() - nodeBlk0[j];
            maxLen = std::max(maxLen, level[j].end - level[j].start);
        }
        const uint32_t nb = (uint32_t)blkNode.size();
        // one upload of the level map: blkNode | blkBegin | nodeStart | nodeEnd | nodeBlk0 | nodeBlkN
        std::vector<uint32_t> map;
        map.insert(map.end(), blkNode.begin(), blkNode.end());
        map.insert(map.end(), blkBegin.begin(), blkBegin.end());
        map.insert(map.end(), nodeStart.begin(), nodeStart.end());
        map.insert(map.end(), nodeEnd.begin(), nodeEnd.end());
        map.insert(map.end(), nodeBlk0.begin(), nodeBlk0.end());
        map.insert(map.end(), nodeBlkN.begin(), nodeBlkN.end());
        if ((rc = uploadVec(mapBuf, map, st))) return rc;
        const uint32_t *mp = (const uint32_t *)mapBuf.ptr;
        LevelMap m{mp, mp + nb, mp + 2 * nb, mp + 2 * nb + nn};
        const uint32_t *nodeBlk0D = mp + 2 * nb + 2 * nn, *nodeBlkND = nodeBlk0D + nn;
        if ((rc = boundsBuf.ensure((size_t)nn * 12 * 4)) || (rc = binsBuf.ensure((size_t)nn * kBinInts * 4)) ||
            (rc = splitBuf.ensure((size_t)nn * 8)) || (rc = cntBuf.ensure((size_t)nb * 4)) ||
            (rc = baseBuf.ensure((size_t)nb * 4)) || (rc = belowBuf.ensure((size_t)nn * 4)) ||
            (rc = rankBuf.ensure((size_t)n * 4)) || (rc = jumpBuf[0].ensure((size_t)n * 4)) ||
            (rc = jumpBuf[1].ensure((size_t)n * 4)))
            return rc;
        int *bounds = (int *)boundsBuf.ptr, *bins = (int *)binsBuf.ptr;
        uint32_t *split = (uint32_t *)splitBuf.ptr;
        const float *bsrc = (const float *)box[buf].ptr, *csrc = (const float *)cent[buf].ptr;
        kInitLevel<<<nn, 64, 0, st>>>(nn, bounds, bins, nullptr);
        if (dim == 3) {
            kLevelBounds<3><<<nb, kLB, 0, st>>>(m, bsrc, csrc, bounds);
            kLevelBins<3><<<nb, kLB, 0, st>>>(m, heuristic, bsrc, csrc, bounds, bins);
            kLevelSplit<3><<<(nn + 63) / 64, 64, 0, st>>>(nn, heuristic, bounds, bins, split);
        } else {
            kLevelBounds<2><<<nb, kLB, 0, st>>>(m, bsrc, csrc, bounds);
            kLevelBins<2><<<nb, kLB, 0, st>>>(m, heuristic, bsrc, csrc, bounds, bins);
            kLevelSplit<2><<<(nn + 63) / 64, 64, 0, st>>>(nn, heuristic, bounds, bins, split);
        }
        kLevelCount<<<nb, kLB, 0, st>>>(m, csrc, split, (uint32_t *)cntBuf.ptr);
        kLevelScan<<<(nn + 63) / 64, 64, 0, st>>>(nn, nodeBlk0D, nodeBlkND, (const uint32_t *)cntBuf.ptr,
                                                  (uint32_t *)baseBuf.ptr, (uint32_t *)belowBuf.ptr);
        kLevelRank<<<nb, kLB, 0, st>>>(m, csrc, split, (const uint32_t *)baseBuf.ptr, (uint32_t *)rankBuf.ptr,
                                       (uint32_t *)jumpBuf[0].ptr);
        int jb = 0;
        for (uint32_t len = 1; len < maxLen; len <<= 1) {  // chains are shorter than the node
            kLevelJump<<<nb, kLB, 0, st>>>(m, (const uint32_t *)jumpBuf[jb].ptr, (uint32_t *)jumpBuf[1 - jb].ptr);
            jb = 1 - jb;
        }
        kLevelGather<<<nb, kLB, 0, st>>>(m, (const uint32_t *)belowBuf.ptr, (const uint32_t *)rankBuf.ptr,
                                         (const uint32_t *)jumpBuf[jb].ptr, bsrc, csrc,
                                         (const uint32_t *)ids[buf].ptr, (float *)box[1 - buf].ptr,
                                         (float *)cent[1 - buf].ptr, (uint32_t *)ids[1 - buf].ptr);
        if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "SAH level pass");
        std::vector<uint32_t> below(nn);
        std::vector<int> hb((size_t)nn * 12);
        if ((e = cudaMemcpyAsync(below.data(), belowBuf.ptr, nn * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hb.data(), bounds, (size_t)nn * 48, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return cudaFail(e, "SAH level read-back");
        std::vector<Pending> next;
        for (uint32_t j = 0; j < nn; j++) {
            const Pending &p = level[j];
            int t = (int)tops.size();
            tops.emplace_back();
            std::memcpy(tops[t].bounds, &hb[(size_t)j * 12], 48);
            if (p.top >= 0) (p.right ? tops[p.top].right : tops[p.top].left) = t;
            const uint32_t len = p.end - p.start;
            uint32_t mid = p.start + below[j];
            if (below[j] == 0 || below[j] == len) mid = p.start + len / 2;
            addChild(p.start, mid, p.depth + 1, t, false, 1 - buf, next);
            addChild(mid, p.end, p.depth + 1, t, true, 1 - buf, next);
        }
        level.swap(next);
        buf = 1 - buf;
    }

    // subtrees of at most kSmall references, one thread each
    const uint32_t nSub = (uint32_t)sStart.size();
    std::vector<uint32_t> sBase(nSub);
    size_t scratchNodes = 0;
    for (uint32_t i = 0; i < nSub; i++) {
        sBase[i] = (uint32_t)scratchNodes;
        scratchNodes += 2 * (size_t)(sEnd[i] - sStart[i]) - 1;
    }
    std::vector<uint32_t> subArr;
    for (auto *v : {&sStart, &sEnd, &sDepth, &sBuf, &sBase}) subArr.insert(subArr.end(), v->begin(), v->end());
    DeviceBuffer subBuf, subNodes, subCount;
    if ((rc = uploadVec(subBuf, subArr, st)) || (rc = subNodes.ensure(scratchNodes * 32)) ||
        (rc = subCount.ensure((size_t)nSub * 4)))
        return rc;
    const uint32_t *sp = (const uint32_t *)subBuf.ptr;
    if (dim == 3)
        kSeqSubtrees<3><<<(nSub + 63) / 64, 64, 0, st>>>(
            heuristic, sp, sp + nSub, sp + 2 * nSub, sp + 3 * nSub, sp + 4 * nSub, nSub, (float *)box[0].ptr,
            (float *)cent[0].ptr, (uint32_t *)ids[0].ptr, (float *)box[1].ptr, (float *)cent[1].ptr,
            (uint32_t *)ids[1].ptr, (unsigned char *)subNodes.ptr, (uint32_t *)subCount.ptr, errorWord);
    else
        kSeqSubtrees<2><<<(nSub + 63) / 64, 64, 0, st>>>(
            heuristic, sp, sp + nSub, sp + 2 * nSub, sp + 3 * nSub, sp + 4 * nSub, nSub, (float *)box[0].ptr,
            (float *)cent[0].ptr, (uint32_t *)ids[0].ptr, (float *)box[1].ptr, (float *)cent[1].ptr,
            (uint32_t *)ids[1].ptr, (unsigned char *)subNodes.ptr, (uint32_t *)subCount.ptr, errorWord);
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "SAH subtrees");
    std::vector<uint32_t> counts(nSub);
    if ((e = cudaMemcpyAsync(counts.data(), subCount.ptr, (size_t)nSub * 4, cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return cudaFail(e, "SAH subtree read-back");

    // pre-order placement: large nodes (records made here) and subtrees (copied)
    std::vector<uint32_t> subPos(nSub);
    std::vector<unsigned char> topRecs;
    std::vector<uint32_t> topPos;
    uint32_t next = 0;
    std::function<uint32_t(int)> place = [&](int t) -> uint32_t {  // returns the subtree's node count
        if (t <= -2) {
            int k = -2 - t;
            subPos[k] = next;
            next += counts[k];
            return counts[k];
        }
        uint32_t me = next++;
        uint32_t nl = place(tops[t].left);
        uint32_t nr = place(tops[t].right);
        float f[6];
        for (int a = 0; a < 6; a++) {
            int v = tops[t].bounds[a];
            int bits = v >= 0 ? v : v ^ 0x7fffffff;
            std::memcpy(&f[a], &bits, 4);
            if (a % 3 >= dim) f[a] = 0.0f;
        }
        uint32_t u[2] = {0u, 1u + nl};
        size_t o = topRecs.size();
        topRecs.resize(o + 32);
        std::memcpy(topRecs.data() + o, f, 24);
        std::memcpy(topRecs.data() + o + 24, u, 8);
        topPos.push_back(me);
        return 1 + nl + nr;
    };
    if (tops.empty()) place(-2);
    else place(0);
    nNodes = next;
    DeviceBuffer posBuf, recBuf, orderBuf;
    if ((rc = nodesOut.ensure((size_t)nNodes * 32)) || (rc = uploadVec(posBuf, subPos, st))) return rc;
    kPlaceSubtrees<<<nSub, 128, 0, st>>>(sp + 4 * nSub, (const uint32_t *)subCount.ptr,
                                         (const uint32_t *)posBuf.ptr, nSub, (const uint4 *)subNodes.ptr,
                                         (uint4 *)nodesOut.ptr);
    if (!topPos.empty()) {
        DeviceBuffer tpBuf;
        if ((rc = uploadVec(recBuf, topRecs, st)) || (rc = uploadVec(tpBuf, topPos, st))) return rc;
        kPlaceNodes<<<((uint32_t)topPos.size() + 127) / 128, 128, 0, st>>>(
            (const unsigned char *)recBuf.ptr, (const uint32_t *)tpBuf.ptr, (uint32_t)topPos.size(),
            (unsigned char *)nodesOut.ptr);
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "SAH node placement");
    }
    // primitives in leaf order
    if ((rc = orderBuf.ensure((size_t)n * 4)) || (rc = primsOut.ensure((size_t)n * (dim == 3 ? 40 : 28))) ||
        (rc = vertsOut.ensure((size_t)n * dim * 4)))
        return rc;
    kFinalOrder<<<nSub, 128, 0, st>>>(sp, sp + nSub, sp + 3 * nSub, nSub, (const uint32_t *)ids[0].ptr,
                                      (const uint32_t *)ids[1].ptr, (uint32_t *)orderBuf.ptr);
    kEmitSahPrimitives<<<g, 256, 0, st>>>(positions, indices, (const uint32_t *)orderBuf.ptr, dim, n,
                                          (unsigned char *)primsOut.ptr, (int32_t *)vertsOut.ptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "SAH emit");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "SAH build");
    return FCPWGB_OK;
}

}  // namespace fcpwgb
