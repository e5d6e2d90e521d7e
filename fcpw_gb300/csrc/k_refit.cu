// Bottom-up BVH refit in one launch.
//
// The reference dispatches one compute pass per tree level with nodeCount
// thread groups each (bvh_interop_structures.h:891-934). Here one thread per
// leaf computes the leaf box (and cone), then climbs towards the root; at every
// inner node the first of the two arriving threads stops and the second one,
// which then knows both children are final, merges them and continues. Arrival
// counts live in a scratch array that must be zero on entry.
//
// Boxes follow the reference exactly (primitive boxes padded by FLT_EPSILON,
// geometry.slang:342-346; merge = component min/max), so refit boxes are
// bit-identical to the CPU refit (bvh.inl:548-599). Leaf cones are built from
// the face normals stored in the silhouette records (bvh.slang:46-98); a leaf
// whose summed axis degenerates keeps halfAngle = pi as the CPU does
// (bvh.inl:505-529). Inner cones use mergeBoundingCones with a unit rotation
// axis (bounding_volumes.h mergeBoundingCones, core.h:129-148).
#include "kernels.h"
#include "silhouette.cuh"

namespace fcpwgb {

// coherent (L2) loads/stores for data written by other threads of this launch
FCPWGB_D float4 ldcg4(const void *p) { return __ldcg(reinterpret_cast<const float4 *>(p)); }

struct RefitBox { float3 pMin, pMax; };

FCPWGB_D void storeBox(unsigned char *nodes, int stride, uint32_t i, const RefitBox &b) {
    float *f = reinterpret_cast<float *>(nodes + (size_t)i * stride);
    f[0] = b.pMin.x; f[1] = b.pMin.y; f[2] = b.pMin.z;
    f[3] = b.pMax.x; f[4] = b.pMax.y; f[5] = b.pMax.z;
}
FCPWGB_D RefitBox loadBoxCoherent(const unsigned char *nodes, int stride, uint32_t i, uint32_t &nPrims,
                                  uint32_t &offset) {
    const unsigned char *p = nodes + (size_t)i * stride;
    float4 a = ldcg4(p), b = ldcg4(p + 16);
    RefitBox r;
    r.pMin = make_float3(a.x, a.y, a.z);
    r.pMax = make_float3(a.w, b.x, b.y);
    nPrims = __float_as_uint(b.z);
    offset = __float_as_uint(b.w);
    return r;
}
struct RefitCone { float3 axis; float halfAngle, radius; };
FCPWGB_D void storeCone(unsigned char *nodes, uint32_t i, const RefitCone &c) {
    float *f = reinterpret_cast<float *>(nodes + (size_t)i * 64 + 32);
    f[0] = c.axis.x; f[1] = c.axis.y; f[2] = c.axis.z; f[3] = c.halfAngle; f[4] = c.radius;
}
FCPWGB_D RefitCone loadConeCoherent(const unsigned char *nodes, uint32_t i, uint32_t &nSil, uint32_t &silOff) {
    const unsigned char *p = nodes + (size_t)i * 64 + 32;
    float4 a = ldcg4(p), b = ldcg4(p + 16);
    RefitCone c;
    c.axis = make_float3(a.x, a.y, a.z);
    c.halfAngle = a.w;
    c.radius = b.x;
    nSil = __float_as_uint(b.y);
    silOff = __float_as_uint(b.z);
    return c;
}

// unit-axis Rodrigues rotation of u towards v (core.h:116-148)
template<int DIM> FCPWGB_D float3 rotateTowards(float3 u, float3 v, float theta) {
    if (DIM == 2) {
        float det = u.x * v.y - u.y * v.x;
        theta *= copysignf(1.0f, det);
        float ct = cosf(theta), st = sinf(theta);
        return make_float3(ct * u.x - st * u.y, st * u.x + ct * u.y, 0.0f);
    }
    float ct = cosf(theta), st = sinf(theta);
    float3 w = normalize3(cross3(u, v));
    float3 o = w * (1.0f - ct);
    float3 r;
    r.x = (ct + o.x * w.x) * u.x + (o.y * w.x - st * w.z) * u.y + (o.z * w.x + st * w.y) * u.z;
    r.y = (o.x * w.y + st * w.z) * u.x + (ct + o.y * w.y) * u.y + (o.z * w.y - st * w.x) * u.z;
    r.z = (o.x * w.z - st * w.y) * u.x + (o.y * w.z + st * w.x) * u.y + (ct + o.z * w.z) * u.z;
    return r;
}

// mergeBoundingCones, bounding_volumes.h / bounding-volumes.slang:256-318
template<int DIM>
FCPWGB_D RefitCone mergeCones(RefitCone a, RefitCone b, float3 oa, float3 ob, float3 o) {
    RefitCone c;
    c.axis = make_float3(0.f, 0.f, 0.f);
    c.halfAngle = kPiF;
    c.radius = 0.0f;
    bool va = a.halfAngle >= 0.0f, vb = b.halfAngle >= 0.0f;
    if (va && vb) {
        float3 da = o - oa, db = o - ob;
        c.radius = sqrtf(fmaxf(a.radius * a.radius + dot3(da, da), b.radius * b.radius + dot3(db, db)));
        if (b.halfAngle > a.halfAngle) { RefitCone t = a; a = b; b = t; }
        float theta = acosf(fmaxf(-1.0f, fminf(1.0f, dot3(a.axis, b.axis))));
        if (fminf(theta + b.halfAngle, kPiF) <= a.halfAngle) {
            c.axis = a.axis;
            c.halfAngle = a.halfAngle;
            return c;
        }
        float oTheta = (a.halfAngle + theta + b.halfAngle) / 2.0f;
        if (oTheta >= kPiF) {
            c.axis = a.axis;
            return c;
        }
        c.axis = rotateTowards<DIM>(a.axis, b.axis, oTheta - a.halfAngle);
        c.halfAngle = oTheta;
    } else if (va) {
        c = a;
    } else if (vb) {
        c = b;
    } else {
        c.halfAngle = -kPiF;
    }
    return c;
}

template<class Prim> FCPWGB_D void primBox(const Prim &p, float3 &lo, float3 &hi);
template<> FCPWGB_D void primBox<TriPrim>(const TriPrim &t, float3 &lo, float3 &hi) {
    float3 e = make_float3(kFltEps, kFltEps, kFltEps);
    lo = fmin3(fmin3(t.pa, t.pb), t.pc) - e;
    hi = fmax3(fmax3(t.pa, t.pb), t.pc) + e;
}
template<> FCPWGB_D void primBox<SegPrim>(const SegPrim &s, float3 &lo, float3 &hi) {
    float3 e = make_float3(kFltEps, kFltEps, 0.0f);
    lo = fmin3(s.pa, s.pb) - e;
    hi = fmax3(s.pa, s.pb) + e;
}

template<class Sil> FCPWGB_D void silNormals(const Sil &s, float3 &n0, float3 &n1, float3 &centroid);
template<> FCPWGB_D void silNormals<EdgeSil>(const EdgeSil &s, float3 &n0, float3 &n1, float3 &c) {
    n0 = s.n0; n1 = s.n1; c = (s.pa + s.pb) * 0.5f;
}
template<> FCPWGB_D void silNormals<VertexSil>(const VertexSil &s, float3 &n0, float3 &n1, float3 &c) {
    n0 = s.n0; n1 = s.n1; c = s.p;
}

template<class Prim, class Sil, int DIM, bool SNCH>
__global__ void __launch_bounds__(256) kRefit(RefitView v) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.nLeaves) return;
    const int stride = SNCH ? 64 : 32;
    uint32_t leaf = v.leaves[t];

    // leaf box
    uint32_t nPrims, offset;
    loadBoxCoherent(v.nodes, stride, leaf, nPrims, offset);
    RefitBox box;
    box.pMin = make_float3(kFltMax, kFltMax, kFltMax);
    box.pMax = make_float3(-kFltMax, -kFltMax, -kFltMax);
    for (uint32_t p = 0; p < nPrims; p++) {
        Prim prim = Prim::load(v.prims, offset + p);
        float3 lo, hi;
        primBox<Prim>(prim, lo, hi);
        box.pMin = fmin3(box.pMin, lo);
        box.pMax = fmax3(box.pMax, hi);
    }
    storeBox(v.nodes, stride, leaf, box);

    if (SNCH) {
        uint32_t nSil, silOff;
        loadConeCoherent(v.nodes, leaf, nSil, silOff);
        float3 centroid = (box.pMin + box.pMax) * 0.5f;
        float3 axis = make_float3(0.f, 0.f, 0.f);
        float radius = 0.0f;
        bool any = false, two = true;
        for (uint32_t k = 0; k < nSil; k++) {
            Sil s = Sil::load(v.sils, silOff + k);
            float3 n0, n1, sc;
            silNormals<Sil>(s, n0, n1, sc);
            axis = axis + n0 + n1;
            radius = fmaxf(radius, len3(sc - centroid));
            two = two && s.hasOne == 0;
            any = true;
        }
        RefitCone cone;
        cone.radius = radius;
        if (!any) {
            cone.axis = make_float3(0.f, 0.f, 0.f);
            cone.halfAngle = -kPiF;
            cone.radius = 0.0f;
        } else if (!two) {
            cone.axis = axis;
            cone.halfAngle = kPiF;
        } else {
            float an = len3(axis);
            if (an > kFltEps) {
                axis = axis / an;
                float ha = 0.0f;
                for (uint32_t k = 0; k < nSil; k++) {
                    Sil s = Sil::load(v.sils, silOff + k);
                    float3 n0, n1, sc;
                    silNormals<Sil>(s, n0, n1, sc);
                    ha = fmaxf(ha, acosf(fmaxf(-1.0f, fminf(1.0f, dot3(axis, n0)))));
                    ha = fmaxf(ha, acosf(fmaxf(-1.0f, fminf(1.0f, dot3(axis, n1)))));
                }
                cone.axis = axis;
                cone.halfAngle = ha;
            } else {
                cone.axis = axis;
                cone.halfAngle = kPiF;
            }
        }
        storeCone(v.nodes, leaf, cone);
    }

    // climb: the second thread to reach a node merges its two children
    __threadfence();
    int32_t node = v.parents[leaf];
    uint32_t guard = 0;
    while (node >= 0 && guard++ < (uint32_t)kStackDepth) {
        uint32_t old = atomicAdd(&v.counters[node], 1u);
        if (old == 0) return;
        __threadfence();
        uint32_t np, off, lnp, loff, rnp, roff;
        loadBoxCoherent(v.nodes, stride, (uint32_t)node, np, off);
        uint32_t li = (uint32_t)node + 1, ri = (uint32_t)node + off;
        RefitBox l = loadBoxCoherent(v.nodes, stride, li, lnp, loff);
        RefitBox r = loadBoxCoherent(v.nodes, stride, ri, rnp, roff);
        RefitBox m;
        m.pMin = fmin3(l.pMin, r.pMin);
        m.pMax = fmax3(l.pMax, r.pMax);
        storeBox(v.nodes, stride, (uint32_t)node, m);
        if (SNCH) {
            uint32_t a0, a1;
            RefitCone lc = loadConeCoherent(v.nodes, li, a0, a1);
            RefitCone rc = loadConeCoherent(v.nodes, ri, a0, a1);
            RefitCone mc = mergeCones<DIM>(lc, rc, (l.pMin + l.pMax) * 0.5f, (r.pMin + r.pMax) * 0.5f,
                                           (m.pMin + m.pMax) * 0.5f);
            storeCone(v.nodes, (uint32_t)node, mc);
        }
        __threadfence();
        node = v.parents[node];
    }
}

cudaError_t launchRefit(const RefitView &v, cudaStream_t s) {
    if (v.nLeaves == 0) return cudaSuccess;
    dim3 g((v.nLeaves + 255) / 256), b(256);
    if (v.dim == 3) {
        if (v.snch) kRefit<TriPrim, EdgeSil, 3, true><<<g, b, 0, s>>>(v);
        else kRefit<TriPrim, EdgeSil, 3, false><<<g, b, 0, s>>>(v);
    } else {
        if (v.snch) kRefit<SegPrim, VertexSil, 2, true><<<g, b, 0, s>>>(v);
        else kRefit<SegPrim, VertexSil, 2, false><<<g, b, 0, s>>>(v);
    }
    return cudaGetLastError();
}

// ----------------------------------------------------- geometry regather
__global__ void kGatherTriangles(const float *pos, const int32_t *pv, uint32_t n, DevTriangle *out) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int a = pv[3 * k], b = pv[3 * k + 1], c = pv[3 * k + 2];
    DevTriangle t = out[k];
    t.pa = make_float3(pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]);
    t.pb = make_float3(pos[3 * b], pos[3 * b + 1], pos[3 * b + 2]);
    t.pc = make_float3(pos[3 * c], pos[3 * c + 1], pos[3 * c + 2]);
    out[k] = t;
}
__global__ void kGatherSegments(const float *pos, const int32_t *pv, uint32_t n, DevSegment2 *out) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int a = pv[2 * k], b = pv[2 * k + 1];
    DevSegment2 s = out[k];
    s.pa = make_float2(pos[2 * a], pos[2 * a + 1]);
    s.pb = make_float2(pos[2 * b], pos[2 * b + 1]);
    out[k] = s;
}
FCPWGB_D float3 ld3(const float *pos, int v) { return make_float3(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]); }
// edge record from its four vertices [opp1, a, b, opp0] (silhouette_edges.inl:45-68)
__global__ void kGatherEdges(const float *pos, const int32_t *sv, uint32_t n, DevEdge *out) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int32_t *v = sv + 4 * k;
    DevEdge e = out[k];
    e.pa = ld3(pos, v[1]);
    e.pb = ld3(pos, v[2]);
    e.n0 = v[3] >= 0 ? normalize3(cross3(e.pb - e.pa, ld3(pos, v[3]) - e.pa)) : make_float3(0.f, 0.f, 0.f);
    e.n1 = v[0] >= 0 ? normalize3(cross3(e.pa - e.pb, ld3(pos, v[0]) - e.pb)) : make_float3(0.f, 0.f, 0.f);
    out[k] = e;
}
// vertex record from [prev, v, next] (silhouette_vertices.inl:34-44)
__global__ void kGatherVertices(const float *pos, const int32_t *sv, uint32_t n, DevVertex2 *out) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int32_t *v = sv + 3 * k;
    DevVertex2 r = out[k];
    float2 p = make_float2(pos[2 * v[1]], pos[2 * v[1] + 1]);
    r.p = p;
    r.n0 = make_float2(0.f, 0.f);
    r.n1 = make_float2(0.f, 0.f);
    if (v[2] >= 0) {
        float2 q = make_float2(pos[2 * v[2]], pos[2 * v[2] + 1]);
        float3 nn = normalize3(make_float3(q.y - p.y, -(q.x - p.x), 0.f));
        r.n0 = make_float2(nn.x, nn.y);
    }
    if (v[0] >= 0) {
        float2 q = make_float2(pos[2 * v[0]], pos[2 * v[0] + 1]);
        float3 nn = normalize3(make_float3(p.y - q.y, -(p.x - q.x), 0.f));
        r.n1 = make_float2(nn.x, nn.y);
    }
    out[k] = r;
}

cudaError_t launchGatherPrimitives(int dim, const float *positions, const int32_t *primVerts, uint32_t nPrims,
                                   unsigned char *prims, cudaStream_t s) {
    if (nPrims == 0) return cudaSuccess;
    dim3 g((nPrims + 255) / 256), b(256);
    if (dim == 3) kGatherTriangles<<<g, b, 0, s>>>(positions, primVerts, nPrims, (DevTriangle *)prims);
    else kGatherSegments<<<g, b, 0, s>>>(positions, primVerts, nPrims, (DevSegment2 *)prims);
    return cudaGetLastError();
}
cudaError_t launchGatherSilhouettes(int dim, const float *positions, const int32_t *silVerts, uint32_t nSils,
                                    unsigned char *sils, cudaStream_t s) {
    if (nSils == 0) return cudaSuccess;
    dim3 g((nSils + 255) / 256), b(256);
    if (dim == 3) kGatherEdges<<<g, b, 0, s>>>(positions, silVerts, nSils, (DevEdge *)sils);
    else kGatherVertices<<<g, b, 0, s>>>(positions, silVerts, nSils, (DevVertex2 *)sils);
    return cudaGetLastError();
}

}  // namespace fcpwgb
