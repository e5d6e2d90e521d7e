// Inside/outside and line-of-sight batches: the reference's Scene<DIM>::
// contains and hasLineOfSight (CPU only there, core/primitive.h:173-207) run
// on the GPU over the transferred binary tree.
//
// contains(x): rays from x along +x and +y, every primitive hit collected
// (the all-hits traversal of bvh.inl:888-1029: no tMax pruning), sorted by
// distance, consecutive duplicates (|d - d'| < 1e-6 and |p - p'|^2 < 1e-6,
// core/interaction.h:20-25,75-94) removed; inside when both counts are odd.
// hasLineOfSight(a, b): an occlusion ray from a towards b with tMax = |b - a|
// (bvh.inl:655-771).
//
// The arithmetic is the CPU code's, rounding for rounding: every operation
// is explicitly rounded (no fused multiply-adds), dot products reduce as
// a0 + (a1 + a2), and the slab test has no parallel-slab guard
// (bounding_volumes.h:99-114, where the GPU shaders add one), so the answers
// equal the reference's bit for bit.
#include "kernels.h"

namespace fcpwgb {

namespace {

constexpr int kMaxHits = 64;  // hits kept per ray; more sets kErrStepBudget and answer 2

FCPWGB_D float cmin(float a, float b) { return b < a ? b : a; }  // std::min
FCPWGB_D float cmax(float a, float b) { return a < b ? b : a; }  // std::max
FCPWGB_D float comp(float3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// BoundingBox::intersect, bounding_volumes.h:99-114
FCPWGB_D bool xboxRay(int dim, float3 pMin, float3 pMax, const DevRay &r, float &tMin) {
    float tn = 0.0f, tf = 0.0f;
    for (int i = 0; i < dim; i++) {
        float t0 = __fmul_rn(__fsub_rn(comp(pMin, i), comp(r.o, i)), comp(r.dInv, i));
        float t1 = __fmul_rn(__fsub_rn(comp(pMax, i), comp(r.o, i)), comp(r.dInv, i));
        float nn = cmin(t0, t1), ff = cmax(t0, t1);
        if (i == 0) {
            tn = nn;
            tf = ff;
        } else {
            tn = cmax(tn, nn);
            tf = cmin(tf, ff);
        }
    }
    float tNearMax = cmax(0.0f, tn), tFarMin = cmin(r.tMax, tf);
    if (tNearMax > tFarMin) return false;
    tMin = tNearMax;
    return true;
}

// Triangle::intersect (Moller-Trumbore), triangles.inl:222-260
FCPWGB_D bool xtriangle(float3 pa, float3 pb, float3 pc, const DevRay &r, float &t, float3 &p) {
    float3 v1 = xsub(pb, pa), v2 = xsub(pc, pa);
    float3 q0 = xcross(r.d, v2);
    float det = xdot(3, v1, q0);
    if (fabsf(det) <= kFltEps) return false;
    float invDet = __fdiv_rn(1.0f, det);
    float3 s = xsub(r.o, pa);
    float v = __fmul_rn(xdot(3, s, q0), invDet);
    if (v < 0.0f || v > 1.0f) return false;
    float3 q = xcross(s, v1);
    float w = __fmul_rn(xdot(3, r.d, q), invDet);
    if (w < 0.0f || __fadd_rn(v, w) > 1.0f) return false;
    t = __fmul_rn(xdot(3, v2, q), invDet);
    if (!(t >= 0.0f && t <= r.tMax)) return false;
    p = xadd(xadd(pa, xmul(v1, v)), xmul(v2, w));
    return true;
}

// LineSegment::intersect, line_segments.inl:140-175
FCPWGB_D bool xsegment(float3 pa, float3 pb, const DevRay &r, float &t, float3 &p) {
    float3 u = xsub(pa, r.o), v = xsub(pb, pa);
    float dv = __fsub_rn(__fmul_rn(r.d.x, v.y), __fmul_rn(r.d.y, v.x));
    if (fabsf(dv) <= kFltEps) return false;
    float ud = __fsub_rn(__fmul_rn(u.x, r.d.y), __fmul_rn(u.y, r.d.x));
    float s = __fdiv_rn(ud, dv);
    if (!(s >= 0.0f && s <= 1.0f)) return false;
    float uv = __fsub_rn(__fmul_rn(u.x, v.y), __fmul_rn(u.y, v.x));
    t = __fdiv_rn(uv, dv);
    if (!(t >= 0.0f && t <= r.tMax)) return false;
    p = xadd(pa, xmul(v, s));
    return true;
}

template<int DIM> FCPWGB_D bool xprimitive(const unsigned char *prims, uint32_t k, const DevRay &r, float &t,
                                           float3 &p) {
    if (DIM == 3) {
        TriPrim tri = TriPrim::load(prims, k);
        return xtriangle(tri.pa, tri.pb, tri.pc, r, t, p);
    }
    SegPrim seg = SegPrim::load(prims, k);
    return xsegment(seg.pa, seg.pb, r, t, p);
}

FCPWGB_D DevRay xray(int dim, float3 o, float3 d, float tMax) {
    DevRay r;
    r.o = o;
    r.d = d;
    r.dInv = make_float3(__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), dim == 3 ? __fdiv_rn(1.0f, d.z) : 0.0f);
    r.tMax = tMax;
    return r;
}

// number of distinct hits along r, or -1 past kMaxHits or the stack depth
template<int DIM, int NODE_STRIDE>
FCPWGB_D int hitCount(const unsigned char *__restrict__ nodes, const unsigned char *__restrict__ prims,
                      const DevRay &r) {
    float ds[kMaxHits];
    float3 ps[kMaxHits];
    int nh = 0;
    uint32_t stack[kStackDepth];
    float tmp;
    NodeBox root = loadNode<NODE_STRIDE>(nodes, 0);
    if (xboxRay(DIM, root.pMin, root.pMax, r, tmp)) {
        int sp = 0;
        stack[0] = 0;
        while (sp >= 0) {
            uint32_t ni = stack[sp--];
            NodeBox node = loadNode<NODE_STRIDE>(nodes, ni);
            if (node.nPrims > 0) {
                for (uint32_t k = 0; k < node.nPrims; k++) {
                    float t;
                    float3 p;
                    if (xprimitive<DIM>(prims, node.offset + k, r, t, p)) {
                        if (nh >= kMaxHits) return -1;
                        ds[nh] = t;
                        ps[nh] = p;
                        nh++;
                    }
                }
            } else {
                uint32_t li = ni + 1, ri = ni + node.offset;
                NodeBox l = loadNode<NODE_STRIDE>(nodes, li), rr = loadNode<NODE_STRIDE>(nodes, ri);
                float t0, t1;
                bool h0 = xboxRay(DIM, l.pMin, l.pMax, r, t0), h1 = xboxRay(DIM, rr.pMin, rr.pMax, r, t1);
                if (sp + 2 >= kStackDepth) return -1;
                // the visiting order does not change the set of hits
                if (h0) stack[++sp] = li;
                if (h1) stack[++sp] = ri;
            }
        }
    }
    for (int i = 1; i < nh; i++) {  // insertion sort by distance
        float d = ds[i];
        float3 p = ps[i];
        int j = i - 1;
        for (; j >= 0 && ds[j] > d; j--) {
            ds[j + 1] = ds[j];
            ps[j + 1] = ps[j];
        }
        ds[j + 1] = d;
        ps[j + 1] = p;
    }
    int count = nh;
    for (int i = 0; i + 1 < nh; i++) {
        float3 dp = xsub(ps[i], ps[i + 1]);
        if (fabsf(__fsub_rn(ds[i], ds[i + 1])) < 1e-6f && xdot(DIM, dp, dp) < 1e-6f) count--;
    }
    return count;
}

// point q at points[stride * q] (3 floats, or the first 3 of a 16 B record);
// with perm non-NULL the points are in sorted order and the answer goes to
// the caller's slot perm[q]
template<int DIM, int NODE_STRIDE>
__global__ void __launch_bounds__(128) kContains(const unsigned char *__restrict__ nodes,
                                                 const unsigned char *__restrict__ prims,
                                                 const float *__restrict__ points, uint32_t stride,
                                                 const uint32_t *__restrict__ perm, uint32_t n, uint32_t *out,
                                                 uint32_t *errorWord) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float *pq = points + (size_t)stride * q;
    float3 x = make_float3(pq[0], pq[1], DIM == 3 ? pq[2] : 0.0f);
    const uint32_t slot = perm ? __ldg(perm + q) : q;
    int h1 = hitCount<DIM, NODE_STRIDE>(nodes, prims, xray(DIM, x, make_float3(1.0f, 0.0f, 0.0f), kFltMax));
    int h2 = hitCount<DIM, NODE_STRIDE>(nodes, prims, xray(DIM, x, make_float3(0.0f, 1.0f, 0.0f), kFltMax));
    if (h1 < 0 || h2 < 0) {
        atomicOr(errorWord, kErrStepBudget);
        out[slot] = 2u;
        return;
    }
    out[slot] = (h1 % 2 == 1 && h2 % 2 == 1) ? 1u : 0u;
}

// points (3 floats each) as 16 B sphere records, the input of the query sort
__global__ void kPackPoints(const float *__restrict__ points, uint32_t n, float4 *__restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float4(points[3 * i], points[3 * i + 1], points[3 * i + 2], 0.0f);
}

template<int DIM, int NODE_STRIDE>
__global__ void __launch_bounds__(128) kLineOfSight(const unsigned char *__restrict__ nodes,
                                                    const unsigned char *__restrict__ prims,
                                                    const float *__restrict__ pa, const float *__restrict__ pb,
                                                    uint32_t n, uint32_t *out, uint32_t *errorWord) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    float3 a = make_float3(pa[3 * q], pa[3 * q + 1], DIM == 3 ? pa[3 * q + 2] : 0.0f);
    float3 b = make_float3(pb[3 * q], pb[3 * q + 1], DIM == 3 ? pb[3 * q + 2] : 0.0f);
    float3 dir = xsub(b, a);
    float dNorm = __fsqrt_rn(xdot(DIM, dir, dir));
    dir = xdiv(dir, dNorm);
    if (DIM == 2) dir.z = 0.0f;
    DevRay r = xray(DIM, a, dir, dNorm);
    bool hit = false;
    uint32_t stackNode[kStackDepth];
    float stackDist[kStackDepth];
    NodeBox root = loadNode<NODE_STRIDE>(nodes, 0);
    float t0;
    if (xboxRay(DIM, root.pMin, root.pMax, r, t0)) {
        int sp = 0;
        stackNode[0] = 0;
        stackDist[0] = t0;
        while (sp >= 0 && !hit) {
            uint32_t ni = stackNode[sp];
            float cur = stackDist[sp];
            sp--;
            if (cur > r.tMax) continue;
            NodeBox node = loadNode<NODE_STRIDE>(nodes, ni);
            if (node.nPrims > 0) {
                for (uint32_t k = 0; k < node.nPrims && !hit; k++) {
                    float t;
                    float3 p;
                    hit = xprimitive<DIM>(prims, node.offset + k, r, t, p);
                }
            } else {
                uint32_t li = ni + 1, ri = ni + node.offset;
                NodeBox l = loadNode<NODE_STRIDE>(nodes, li), rr = loadNode<NODE_STRIDE>(nodes, ri);
                float l0, r0;
                bool h0 = xboxRay(DIM, l.pMin, l.pMax, r, l0), h1 = xboxRay(DIM, rr.pMin, rr.pMax, r, r0);
                if (sp + 2 >= kStackDepth) {
                    atomicOr(errorWord, kErrStackOverflow);
                    break;
                }
                if (h0 && h1) {
                    uint32_t closer = li, other = ri;
                    float dc = l0, dother = r0;
                    if (r0 < l0) {
                        closer = ri;
                        other = li;
                        dc = r0;
                        dother = l0;
                    }
                    ++sp; stackNode[sp] = other; stackDist[sp] = dother;
                    ++sp; stackNode[sp] = closer; stackDist[sp] = dc;
                } else if (h0 || h1) {
                    ++sp;
                    stackNode[sp] = h0 ? li : ri;
                    stackDist[sp] = h0 ? l0 : r0;
                }
            }
        }
    }
    out[q] = hit ? 0u : 1u;
}

}  // namespace

cudaError_t launchContains(const SceneView &v, const float *points, uint32_t stride, const uint32_t *perm,
                           uint32_t n, uint32_t *out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 g((n + 127) / 128), b(128);
    if (v.dim == 3) {
        if (v.snch) kContains<3, 64><<<g, b, 0, s>>>(v.nodes, v.prims, points, stride, perm, n, out, v.errorWord);
        else kContains<3, 32><<<g, b, 0, s>>>(v.nodes, v.prims, points, stride, perm, n, out, v.errorWord);
    } else {
        if (v.snch) kContains<2, 64><<<g, b, 0, s>>>(v.nodes, v.prims, points, stride, perm, n, out, v.errorWord);
        else kContains<2, 32><<<g, b, 0, s>>>(v.nodes, v.prims, points, stride, perm, n, out, v.errorWord);
    }
    return cudaGetLastError();
}

cudaError_t launchPackPoints(const float *points, uint32_t n, DevSphere *out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    kPackPoints<<<(n + 255) / 256, 256, 0, s>>>(points, n, reinterpret_cast<float4 *>(out));
    return cudaGetLastError();
}

cudaError_t launchLineOfSight(const SceneView &v, const float *a, const float *b, uint32_t n, uint32_t *out,
                              cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 g((n + 127) / 128), bl(128);
    if (v.dim == 3) {
        if (v.snch) kLineOfSight<3, 64><<<g, bl, 0, s>>>(v.nodes, v.prims, a, b, n, out, v.errorWord);
        else kLineOfSight<3, 32><<<g, bl, 0, s>>>(v.nodes, v.prims, a, b, n, out, v.errorWord);
    } else {
        if (v.snch) kLineOfSight<2, 64><<<g, bl, 0, s>>>(v.nodes, v.prims, a, b, n, out, v.errorWord);
        else kLineOfSight<2, 32><<<g, bl, 0, s>>>(v.nodes, v.prims, a, b, n, out, v.errorWord);
    }
    return cudaGetLastError();
}

}  // namespace fcpwgb
