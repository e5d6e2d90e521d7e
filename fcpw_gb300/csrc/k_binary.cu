// Query kernels over the binary (reference-layout) BVH: one thread per query,
// depth-first with a 64-entry per-thread stack, exactly the traversal order of
// the reference GPU path (include/fcpw/gpu/bvh.slang). These are the parity
// kernels; the wide/quantised kernels in k_wide.cu are the fast path.
#include "kernels.h"
#include "binary_queries.cuh"
#include "silhouette.cuh"

namespace fcpwgb {

// ------------------------------------------------------- closest point
// Bvh.findClosestPoint, bvh.slang:395-502
// With COUNT, per-launch totals of popped nodes, expanded inner nodes and
// primitive tests are accumulated into stats[0..2] (traversal statistics mode).
template<class Prim, int NODE_STRIDE, bool COUNT = false>
__global__ void __launch_bounds__(256) kClosestPointBinary(const unsigned char *__restrict__ nodes,
                                                           const unsigned char *__restrict__ prims,
                                                           const DevSphere *__restrict__ spheres,
                                                           DevInteraction *__restrict__ out, uint32_t n,
                                                           int recordNormal, uint32_t *errorWord,
                                                           unsigned long long *stats = nullptr) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    float4 s4 = ldg4(spheres + q);
    float3 c = make_float3(s4.x, s4.y, s4.z);
    float r2 = s4.w;
    DevInteraction best = defaultInteraction();
    uint32_t selected = kUintMax;

    uint32_t stack[kStackDepth];
    uint32_t cPop = 0, cInner = 0, cPrim = 0;
    NodeBox root = loadNode<NODE_STRIDE>(nodes, 0);
    float d2Min, d2Max;
    boxSphereDist(root.pMin, root.pMax, c, d2Min, d2Max);
    if (d2Min <= r2) {
        r2 = fminf(r2, d2Max);
        stack[0] = 0;
        int sp = 0;
        while (sp >= 0) {
            uint32_t ni = stack[sp--];
            NodeBox node = loadNode<NODE_STRIDE>(nodes, ni);
            if (COUNT) cPop++;
            if (!(boxSphereD2Min(node.pMin, node.pMax, c) <= r2)) continue;
            if (node.nPrims > 0) {
                if (COUNT) cPrim += node.nPrims;
                for (uint32_t p = 0; p < node.nPrims; p++) {
                    uint32_t pi = node.offset + p;
                    Prim prim = Prim::load(prims, pi);
                    float3 pt;
                    float2 uv;
                    float d = prim.closestPoint(c, pt, uv);
                    if (d * d <= r2) {
                        r2 = fminf(r2, d * d);
                        best.p = pt;
                        best.n = make_float3(0.f, 0.f, 0.f);
                        best.uv = uv;
                        best.d = d;
                        best.index = prim.index;
                        selected = pi;
                    }
                }
            } else {
                if (COUNT) cInner++;
                uint32_t li = ni + 1, ri = ni + node.offset;
                NodeBox l = loadNode<NODE_STRIDE>(nodes, li);
                NodeBox r = loadNode<NODE_STRIDE>(nodes, ri);
                float l0, l1, r0, r1;
                boxSphereDist(l.pMin, l.pMax, c, l0, l1);
                bool hitL = l0 <= r2;
                r2 = fminf(r2, l1);
                boxSphereDist(r.pMin, r.pMax, c, r0, r1);
                bool hitR = r0 <= r2;
                r2 = fminf(r2, r1);
                if (hitL && hitR) {
                    uint32_t closer = li, other = ri;
                    if (r0 < l0) { closer = ri; other = li; }
                    if (sp + 2 >= kStackDepth) { atomicOr(errorWord, kErrStackOverflow); break; }
                    stack[++sp] = other;
                    stack[++sp] = closer;
                } else if (hitL || hitR) {
                    if (sp + 1 >= kStackDepth) { atomicOr(errorWord, kErrStackOverflow); break; }
                    stack[++sp] = hitL ? li : ri;
                }
            }
        }
    }
    if (selected != kUintMax && recordNormal) best.n = Prim::load(prims, selected).normal();
    out[q] = best;
    if (COUNT) {
        atomicAdd(stats + 0, (unsigned long long)cPop);
        atomicAdd(stats + 1, (unsigned long long)cInner);
        atomicAdd(stats + 2, (unsigned long long)cPrim);
    }
}

// ----------------------------------------------------------------- rays
// Bvh.intersect(ray), bvh.slang:144-254
template<class Prim, int NODE_STRIDE>
__global__ void __launch_bounds__(256) kRayBinary(const unsigned char *__restrict__ nodes,
                                                  const unsigned char *__restrict__ prims,
                                                  const DevRay *__restrict__ rays,
                                                  DevInteraction *__restrict__ out, uint32_t n, int occl,
                                                  uint32_t *errorWord) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const unsigned char *rp = reinterpret_cast<const unsigned char *>(rays + q);
    float2 a = ldg2(rp), b = ldg2(rp + 8), cc = ldg2(rp + 16), d = ldg2(rp + 24), e = ldg2(rp + 32);
    DevRay r;
    r.o = make_float3(a.x, a.y, b.x);
    r.d = make_float3(b.y, cc.x, cc.y);
    r.dInv = make_float3(d.x, d.y, e.x);
    r.tMax = e.y;

    DevInteraction best = defaultInteraction();
    uint32_t stackNode[kStackDepth];
    float stackDist[kStackDepth];
    NodeBox root = loadNode<NODE_STRIDE>(nodes, 0);
    float t0, t1;
    if (boxRayIntersect(root.pMin, root.pMax, r, t0, t1)) {
        stackNode[0] = 0;
        stackDist[0] = t0;
        int sp = 0;
        while (sp >= 0) {
            uint32_t ni = stackNode[sp];
            float dist = stackDist[sp];
            sp--;
            if (dist > r.tMax) continue;
            NodeBox node = loadNode<NODE_STRIDE>(nodes, ni);
            if (node.nPrims > 0) {
                bool done = false;
                for (uint32_t p = 0; p < node.nPrims; p++) {
                    Prim prim = Prim::load(prims, node.offset + p);
                    DevInteraction c = defaultInteraction();
                    if (prim.intersect(r, occl != 0, c)) {
                        c.index = prim.index;
                        if (occl) {
                            best.index = c.index;
                            done = true;
                            break;
                        }
                        r.tMax = fminf(r.tMax, c.d);
                        best = c;
                    }
                }
                if (done) break;
            } else {
                uint32_t li = ni + 1, ri = ni + node.offset;
                NodeBox l = loadNode<NODE_STRIDE>(nodes, li);
                NodeBox rr = loadNode<NODE_STRIDE>(nodes, ri);
                float l0, l1, r0, r1;
                bool hitL = boxRayIntersect(l.pMin, l.pMax, r, l0, l1);
                bool hitR = boxRayIntersect(rr.pMin, rr.pMax, r, r0, r1);
                if (hitL && hitR) {
                    uint32_t closer = li, other = ri;
                    float dc = l0, dother = r0;
                    if (r0 < l0) { closer = ri; other = li; dc = r0; dother = l0; }
                    if (sp + 2 >= kStackDepth) { atomicOr(errorWord, kErrStackOverflow); break; }
                    ++sp; stackNode[sp] = other; stackDist[sp] = dother;
                    ++sp; stackNode[sp] = closer; stackDist[sp] = dc;
                } else if (hitL || hitR) {
                    if (sp + 1 >= kStackDepth) { atomicOr(errorWord, kErrStackOverflow); break; }
                    ++sp;
                    stackNode[sp] = hitL ? li : ri;
                    stackDist[sp] = hitL ? l0 : r0;
                }
            }
        }
    }
    out[q] = best;
}

// ------------------------------------------------- sphere sampling
// Bvh.intersect(sphere, randNums) with constant branch weights, bvh.slang:257-392
// (sphereSampleBinary, binary_queries.cuh)
template<class Prim, int NODE_STRIDE>
__global__ void __launch_bounds__(256) kSphereSampleBinary(const unsigned char *__restrict__ nodes,
                                                           const unsigned char *__restrict__ prims,
                                                           const DevSphere *__restrict__ spheres,
                                                           const float3 *__restrict__ randNums,
                                                           DevInteraction *__restrict__ out, uint32_t n,
                                                           uint32_t depthLimit, uint32_t *errorWord) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    float4 s4 = ldg4(spheres + q);
    DevInteraction best;
    sphereSampleBinary<Prim, NODE_STRIDE>(nodes, prims, make_float3(s4.x, s4.y, s4.z), s4.w, randNums[q], depthLimit,
                                          errorWord, best);
    out[q] = best;
}

// ------------------------------------------- closest silhouette point
// Bvh.findClosestSilhouettePoint, bvh.slang:505-646 (SNCH nodes only; silhouetteBinary,
// binary_queries.cuh)
template<class Sil, int DIM>
__global__ void __launch_bounds__(256) kSilhouetteBinary(const unsigned char *__restrict__ nodes,
                                                         const unsigned char *__restrict__ sils,
                                                         const DevSphere *__restrict__ spheres,
                                                         const uint32_t *__restrict__ flip,
                                                         const uint32_t *__restrict__ perm,
                                                         DevInteraction *__restrict__ out, uint32_t n,
                                                         float sqMinR, float precision, uint32_t *errorWord) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const uint32_t src = perm ? __ldg(perm + q) : q;  // sorted queries: the caller's slot
    float4 s4 = ldg4(spheres + q);
    float r2 = s4.w;
    DevInteraction best;
    silhouetteBinary<Sil, DIM>(nodes, sils, make_float3(s4.x, s4.y, s4.z), r2, __ldg(flip + src) != 0, sqMinR,
                               precision, errorWord, best);
    out[src] = best;
}

// ------------------------------------------------------------ launchers
static inline uint32_t blocksFor(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

cudaError_t launchClosestPointBinary(const SceneView &v, const DevSphere *spheres, DevInteraction *out,
                                     uint32_t n, int recordNormal, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 g(blocksFor(n, 256)), b(256);
    if (v.dim == 3) {
        if (v.snch) kClosestPointBinary<TriPrim, 64><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, recordNormal, v.errorWord);
        else kClosestPointBinary<TriPrim, 32><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, recordNormal, v.errorWord);
    } else {
        if (v.snch) kClosestPointBinary<SegPrim, 64><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, recordNormal, v.errorWord);
        else kClosestPointBinary<SegPrim, 32><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, recordNormal, v.errorWord);
    }
    return cudaGetLastError();
}

cudaError_t launchClosestPointBinaryStats(const SceneView &v, const DevSphere *spheres, DevInteraction *out,
                                          uint32_t n, unsigned long long *stats, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 g(blocksFor(n, 256)), b(256);
    if (v.dim == 3) {
        if (v.snch) kClosestPointBinary<TriPrim, 64, true><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, 0, v.errorWord, stats);
        else kClosestPointBinary<TriPrim, 32, true><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, 0, v.errorWord, stats);
    } else {
        if (v.snch) kClosestPointBinary<SegPrim, 64, true><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, 0, v.errorWord, stats);
        else kClosestPointBinary<SegPrim, 32, true><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, out, n, 0, v.errorWord, stats);
    }
    return cudaGetLastError();
}

cudaError_t launchRayBinary(const SceneView &v, const DevRay *rays, DevInteraction *out, uint32_t n, int occl,
                            cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 g(blocksFor(n, 256)), b(256);
    if (v.dim == 3) {
        if (v.snch) kRayBinary<TriPrim, 64><<<g, b, 0, s>>>(v.nodes, v.prims, rays, out, n, occl, v.errorWord);
        else kRayBinary<TriPrim, 32><<<g, b, 0, s>>>(v.nodes, v.prims, rays, out, n, occl, v.errorWord);
    } else {
        if (v.snch) kRayBinary<SegPrim, 64><<<g, b, 0, s>>>(v.nodes, v.prims, rays, out, n, occl, v.errorWord);
        else kRayBinary<SegPrim, 32><<<g, b, 0, s>>>(v.nodes, v.prims, rays, out, n, occl, v.errorWord);
    }
    return cudaGetLastError();
}

cudaError_t launchSphereSampleBinary(const SceneView &v, const DevSphere *spheres, const float3 *randNums,
                                     DevInteraction *out, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 g(blocksFor(n, 256)), b(256);
    uint32_t lim = v.maxDepth + 1;
    if (v.dim == 3) {
        if (v.snch) kSphereSampleBinary<TriPrim, 64><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, randNums, out, n, lim, v.errorWord);
        else kSphereSampleBinary<TriPrim, 32><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, randNums, out, n, lim, v.errorWord);
    } else {
        if (v.snch) kSphereSampleBinary<SegPrim, 64><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, randNums, out, n, lim, v.errorWord);
        else kSphereSampleBinary<SegPrim, 32><<<g, b, 0, s>>>(v.nodes, v.prims, spheres, randNums, out, n, lim, v.errorWord);
    }
    return cudaGetLastError();
}

cudaError_t launchSilhouetteBinary(const SceneView &v, const DevSphere *spheres, const uint32_t *flip,
                                   const uint32_t *perm, DevInteraction *out, uint32_t n, float sqMinR,
                                   float precision, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 g(blocksFor(n, 256)), b(256);
    if (v.dim == 3) kSilhouetteBinary<EdgeSil, 3><<<g, b, 0, s>>>(v.nodes, v.sils, spheres, flip, perm, out, n, sqMinR, precision, v.errorWord);
    else kSilhouetteBinary<VertexSil, 2><<<g, b, 0, s>>>(v.nodes, v.sils, spheres, flip, perm, out, n, sqMinR, precision, v.errorWord);
    return cudaGetLastError();
}

// default results for queries when the scene has no silhouettes
__global__ void kFillDefault(DevInteraction *out, uint32_t n) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) out[q] = defaultInteraction();
}
cudaError_t launchFillDefault(DevInteraction *out, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    kFillDefault<<<blocksFor(n, 256), 256, 0, s>>>(out, n);
    return cudaGetLastError();
}

}  // namespace fcpwgb
