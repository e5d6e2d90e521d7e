// Scenes of several objects and instanced objects on the GPU.
//
// The reference's CPU Scene<DIM> takes several objects and, per object, a
// list of instance transforms (Scene::setObjectCount / setObjectInstanceTransforms,
// fcpw.h:29-70). Scene::build (fcpw.inl:1053-1102) makes one BVH per object,
// wraps every instance of a transformed object in a TransformedAggregate
// (core/primitive.h:289-478), and builds a top-level BVH over the instances
// with the same binned SAH (bvh.inl:40-234), whose leaves are aggregates. Its
// GPU path takes single-object scenes only (fcpw_gpu.h:17-20; the Slang
// TransformedAggregate, aggregate.slang:45-145, is never bound).
//
// Here the same structure runs on the device. Every object keeps its own
// scene (binary tree, 4-wide tree with the configured box precision, 48 B
// triangles or 24 B segments); the instances are 112 B records holding the
// affine transform t, its inverse and the object; the top-level tree is the
// 32 B interop layout with one instance index per leaf reference. A query
// walks the top-level tree in the reference's CPU order (aggregate leaves of
// bvh.inl:1291-1418 and 655-771), takes each instance's query to object space
// (BoundingSphere / Ray ::transform, bounding_volumes.h:13-24, ray.h:19-25),
// walks the object's wide tree, and maps the result back
// (Interaction::applyTransform, interaction.h:52-60); an object without
// transforms is walked as it is. Transform arithmetic is that of the affine
// Transform the reference's CPU build was checked with: row i of t*p is
// t(i,D) + t(i,0)*p0 + t(i,1)*p1 [+ t(i,2)*p2], summed in that order, without
// fused multiply-adds; inverses are Gauss-Jordan eliminations in double.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "host_bvh.h"
#include "k_wide.cuh"
#include "kernels.h"
#include "scene.h"

using namespace fcpwgb;

// ---------------------------------------------------------------- host side
struct fcpwgb_cpu_instances {
    int dim = 3;
    std::vector<const fcpwgb_cpu_bvh *> objects;  // borrowed: alive until the transfer
    std::vector<uint32_t> object, transformed;
    std::vector<float> t, ti;                     // 12 per instance: rows of [A | b] (2D: rows 0-1, z unused)
    std::vector<float> boxes;                     // 6 per instance, world space
    std::unique_ptr<HostBvh> top;                 // null for a single instance (no top-level tree)
};

namespace fcpwgb {

struct DevInstance {
    float t[12];
    float ti[12];
    uint32_t object, transformed, pad0, pad1;
};
static_assert(sizeof(DevInstance) == 112, "instance record");

struct DevObject {
    const unsigned char *nodes;  // 4-wide records
    const unsigned char *prims;  // Tri48 / Seg24 records
};

struct InstancedState {
    int dim = 3;
    uint32_t nInstances = 0, nTopNodes = 0;
    std::vector<fcpwgb_gpu_scene *> objects;
    std::vector<uint32_t> instObject;
    DeviceBuffer topNodes, topRefs, instances, objectTable, instOut;
    int tableBits = -1, tableLeaf = -1;
    float worldBox[6] = {0, 0, 0, 0, 0, 0};
    ~InstancedState() {
        for (auto *o : objects) fcpwgb_gpu_scene_destroy(o);
    }
};

namespace {

// (D+1) x (D+1) affine inverse by Gauss-Jordan elimination with partial
// pivoting in double; false when singular
bool invertAffine(int dim, const double *m, double *inv) {
    const int n = dim + 1;
    double a[16], r[16];
    for (int i = 0; i < n * n; i++) {
        a[i] = m[i];
        r[i] = (i / n == i % n) ? 1.0 : 0.0;
    }
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int row = c + 1; row < n; row++)
            if (std::fabs(a[row * n + c]) > std::fabs(a[p * n + c])) p = row;
        for (int k = 0; k < n; k++) {
            std::swap(a[p * n + k], a[c * n + k]);
            std::swap(r[p * n + k], r[c * n + k]);
        }
        double d = a[c * n + c];
        if (d == 0.0 || !std::isfinite(d)) return false;
        for (int k = 0; k < n; k++) {
            a[c * n + k] /= d;
            r[c * n + k] /= d;
        }
        for (int row = 0; row < n; row++) {
            if (row == c) continue;
            double f = a[row * n + c];
            for (int k = 0; k < n; k++) {
                a[row * n + k] -= f * a[c * n + k];
                r[row * n + k] -= f * r[c * n + k];
            }
        }
    }
    for (int i = 0; i < n * n; i++) inv[i] = r[i];
    return true;
}

// t*p with the reference order: translation first, then the columns
void xfPointHost(int dim, const float *m12, const float *p, float *out) {
    for (int i = 0; i < dim; i++) {
        float acc = m12[i * 4 + 3];
        for (int k = 0; k < dim; k++) acc += m12[i * 4 + k] * p[k];
        out[i] = acc;
    }
}

int heuristicOf(int aggregateType, Heuristic &h) {
    switch (aggregateType) {
        case FCPWGB_AGGREGATE_BVH_LONGEST_AXIS: h = Heuristic::LongestAxisCenter; return 0;
        case FCPWGB_AGGREGATE_BVH_OVERLAP_SURFACE: h = Heuristic::OverlapSurfaceArea; return 0;
        case FCPWGB_AGGREGATE_BVH_SURFACE_AREA: h = Heuristic::SurfaceArea; return 0;
        case FCPWGB_AGGREGATE_BVH_OVERLAP_VOLUME: h = Heuristic::OverlapVolume; return 0;
        case FCPWGB_AGGREGATE_BVH_VOLUME: h = Heuristic::Volume; return 0;
        default: return setError(FCPWGB_ERR_UNSUPPORTED, "instanced scenes need a BVH aggregate type (Bvh_*)");
    }
}

}  // namespace
}  // namespace fcpwgb

extern "C" int fcpwgb_cpu_instances_build(int dim, int aggregate_type, const fcpwgb_cpu_bvh *const *objects,
                                          uint32_t n_objects, const uint32_t *instance_objects,
                                          const float *transforms, const uint32_t *transformed,
                                          uint32_t n_instances, fcpwgb_cpu_instances **out) {
    if (!out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (dim != 2 && dim != 3) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
    if (!objects || n_objects == 0) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "at least one object is required");
    if (!instance_objects || n_instances == 0)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "at least one instance is required");
    Heuristic h;
    int rc = heuristicOf(aggregate_type, h);
    if (rc) return rc;
    for (uint32_t k = 0; k < n_objects; k++) {
        if (!objects[k] || !objects[k]->bvh) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL object");
        if (objects[k]->bvh->dim() != dim)
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "an object's dimension differs from the scene's");
    }
    std::unique_ptr<fcpwgb_cpu_instances> r(new fcpwgb_cpu_instances);
    r->dim = dim;
    r->objects.assign(objects, objects + n_objects);
    r->object.resize(n_instances);
    r->transformed.resize(n_instances);
    r->t.assign((size_t)n_instances * 12, 0.0f);
    r->ti.assign((size_t)n_instances * 12, 0.0f);
    r->boxes.resize((size_t)n_instances * 6);
    std::vector<float> centroids((size_t)n_instances * 3, 0.0f);
    const int D = dim;
    for (uint32_t i = 0; i < n_instances; i++) {
        if (instance_objects[i] >= n_objects)
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "instance object index out of range");
        const HostBvh &ob = *objects[instance_objects[i]]->bvh;
        r->object[i] = instance_objects[i];
        bool tr = transforms && (!transformed || transformed[i] != 0);
        r->transformed[i] = tr ? 1u : 0u;
        float lo[3], hi[3], c[3];
        ob.rootBox(lo, hi);
        ob.primitiveCentroidMean(c);
        float *t12 = &r->t[(size_t)i * 12], *ti12 = &r->ti[(size_t)i * 12];
        if (!tr) {
            for (int a = 0; a < 3; a++) {
                t12[a * 4 + a] = 1.0f;
                ti12[a * 4 + a] = 1.0f;
            }
            for (int a = 0; a < 3; a++) {
                r->boxes[(size_t)i * 6 + a] = a < D ? lo[a] : 0.0f;
                r->boxes[(size_t)i * 6 + 3 + a] = a < D ? hi[a] : 0.0f;
                centroids[(size_t)i * 3 + a] = a < D ? c[a] : 0.0f;
            }
            continue;
        }
        // rows of [A | b] (D x (D+1) floats per instance) into the 3x4 layout
        const float *src = transforms + (size_t)i * D * (D + 1);
        double full[16], inv[16];
        const int n = D + 1;
        for (int a = 0; a < n * n; a++) full[a] = 0.0;
        for (int a = 0; a < D; a++) {
            for (int b = 0; b <= D; b++) {
                float v = src[a * (D + 1) + b];
                if (!std::isfinite(v)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "non-finite instance transform");
                full[a * n + b] = (double)v;
                t12[a * 4 + (b == D ? 3 : b)] = v;
            }
        }
        full[D * n + D] = 1.0;
        if (!invertAffine(D, full, inv)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "singular instance transform");
        for (int a = 0; a < D; a++)
            for (int b = 0; b <= D; b++) ti12[a * 4 + (b == D ? 3 : b)] = (float)inv[a * n + b];
        if (D == 2) {  // unused z row / column: identity, so 3D code paths see z unchanged
            t12[2 * 4 + 2] = 1.0f;
            ti12[2 * 4 + 2] = 1.0f;
        }
        // BoundingBox::transform (bounding_volumes.h:184-200): every corner mapped and
        // included (expandToInclude pads each by FLT_EPSILON); centroid t * c
        float bl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int corner = 0; corner < (1 << D); corner++) {
            float p[3], q[3];
            int temp = corner;
            for (int a = 0; a < D; a++) {
                p[a] = temp % 2 == 0 ? lo[a] : hi[a];
                temp /= 2;
            }
            xfPointHost(D, t12, p, q);
            for (int a = 0; a < D; a++) {
                float l = q[a] - FLT_EPSILON, u = q[a] + FLT_EPSILON;
                bl[a] = l < bl[a] ? l : bl[a];
                bh[a] = bh[a] < u ? u : bh[a];
            }
        }
        float tc[3] = {0, 0, 0};
        xfPointHost(D, t12, c, tc);
        for (int a = 0; a < 3; a++) {
            r->boxes[(size_t)i * 6 + a] = a < D ? bl[a] : 0.0f;
            r->boxes[(size_t)i * 6 + 3 + a] = a < D ? bh[a] : 0.0f;
            centroids[(size_t)i * 3 + a] = a < D ? tc[a] : 0.0f;
        }
    }
    if (n_instances > 1) {
        try {
            r->top = HostBvh::fromBoxes(dim, r->boxes.data(), centroids.data(), n_instances, h);
        } catch (const std::exception &e) {
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, e.what());
        }
    }
    *out = r.release();
    return FCPWGB_OK;
}

extern "C" void fcpwgb_cpu_instances_destroy(fcpwgb_cpu_instances *inst) { delete inst; }

extern "C" int fcpwgb_cpu_instances_export(const fcpwgb_cpu_instances *inst, void *top_nodes, uint32_t *top_refs,
                                           float *instance_matrices, uint32_t *n_top_nodes) {
    if (!inst) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL instances");
    uint32_t nn = inst->top ? inst->top->nNodes() : 0u;
    if (n_top_nodes) *n_top_nodes = nn;
    if (top_nodes && inst->top) inst->top->exportNodes(top_nodes);
    if (top_refs && inst->top)
        for (size_t k = 0; k < inst->top->primOrder().size(); k++) top_refs[k] = (uint32_t)inst->top->primOrder()[k];
    if (instance_matrices) {
        size_t n = inst->object.size();
        for (size_t i = 0; i < n; i++) {
            std::memcpy(instance_matrices + i * 24, &inst->t[i * 12], 12 * sizeof(float));
            std::memcpy(instance_matrices + i * 24 + 12, &inst->ti[i * 12], 12 * sizeof(float));
        }
    }
    return FCPWGB_OK;
}

// --------------------------------------------------------------- device side
namespace fcpwgb {
namespace {

FCPWGB_D float3 xfPoint(int dim, const float *__restrict__ m, float3 p) {
    float r[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float acc = m[i * 4 + 3];
        acc = __fadd_rn(acc, __fmul_rn(m[i * 4 + 0], p.x));
        acc = __fadd_rn(acc, __fmul_rn(m[i * 4 + 1], p.y));
        if (dim == 3) acc = __fadd_rn(acc, __fmul_rn(m[i * 4 + 2], p.z));
        r[i] = acc;
    }
    return make_float3(r[0], r[1], dim == 3 ? r[2] : 0.0f);
}

FCPWGB_D float xdot3(int dim, float3 a, float3 b) {
    return dim == 3 ? __fadd_rn(__fmul_rn(a.x, b.x), __fadd_rn(__fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)))
                    : __fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
FCPWGB_D float3 xsub3(float3 a, float3 b) {
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}

// BoundingSphere::transform: radius measured along +x
FCPWGB_D float xfR2(int dim, const float *__restrict__ m, float3 c, float3 tc, float r2) {
    if (!(r2 < kFltMax)) return kFltMax;
    float3 e = make_float3(__fadd_rn(c.x, __fsqrt_rn(r2)), __fadd_rn(c.y, 0.0f), __fadd_rn(c.z, 0.0f));
    float3 d = xsub3(xfPoint(dim, m, e), tc);
    return xdot3(dim, d, d);
}

// Interaction::applyTransform: p to world space, distance to the query
// recomputed, normal through the transposed inverse and renormalised
FCPWGB_D void xfInteraction(int dim, const DevInstance &I, float3 query, DevInteraction &c) {
    c.p = xfPoint(dim, I.t, c.p);
    float3 d = xsub3(c.p, query);
    c.d = __fsqrt_rn(xdot3(dim, d, d));
    float r[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float acc = 0.0f;
        acc = __fadd_rn(acc, __fmul_rn(I.ti[0 * 4 + i], c.n.x));
        acc = __fadd_rn(acc, __fmul_rn(I.ti[1 * 4 + i], c.n.y));
        if (dim == 3) acc = __fadd_rn(acc, __fmul_rn(I.ti[2 * 4 + i], c.n.z));
        r[i] = acc;
    }
    float3 n = make_float3(r[0], r[1], dim == 3 ? r[2] : 0.0f);
    float z = xdot3(dim, n, n);
    if (z > 0.0f) {
        float s = __fsqrt_rn(z);
        n = make_float3(__fdiv_rn(n.x, s), __fdiv_rn(n.y, s), __fdiv_rn(n.z, s));
    }
    c.n = n;
}

// Ray::transform: origin and a point along the ray mapped, direction renormalised
FCPWGB_D DevRay xfRay(int dim, const float *__restrict__ m, const DevRay &r) {
    DevRay o;
    o.o = xfPoint(dim, m, r.o);
    float s = r.tMax < kFltMax ? r.tMax : 1.0f;
    float3 end = make_float3(__fadd_rn(r.o.x, __fmul_rn(r.d.x, s)), __fadd_rn(r.o.y, __fmul_rn(r.d.y, s)),
                             __fadd_rn(r.o.z, __fmul_rn(r.d.z, s)));
    float3 td = xsub3(xfPoint(dim, m, end), o.o);
    float nrm = __fsqrt_rn(xdot3(dim, td, td));
    o.d = make_float3(__fdiv_rn(td.x, nrm), __fdiv_rn(td.y, nrm), __fdiv_rn(td.z, nrm));
    o.dInv = make_float3(__frcp_rn(o.d.x), __frcp_rn(o.d.y), __frcp_rn(o.d.z));
    o.tMax = r.tMax < kFltMax ? nrm : kFltMax;
    return o;
}

// sphere-box distances in the reference's order (bounding_volumes.h:62-90)
FCPWGB_D void xboxSphere(int dim, float3 pMin, float3 pMax, float3 c, float &d2Min, float &d2Max) {
    float3 u = xsub3(pMin, c), v = xsub3(c, pMax);
    float3 a = make_float3(fmaxf(fmaxf(u.x, v.x), 0.0f), fmaxf(fmaxf(u.y, v.y), 0.0f), fmaxf(fmaxf(u.z, v.z), 0.0f));
    float3 b = make_float3(fminf(u.x, v.x), fminf(u.y, v.y), fminf(u.z, v.z));
    d2Min = xdot3(dim, a, a);
    d2Max = xdot3(dim, b, b);
}

// ray-box slab test of the reference CPU (bounding_volumes.h:99-114)
FCPWGB_D bool xboxRayCpu(int dim, float3 pMin, float3 pMax, const DevRay &r, float &tMin) {
    float tn = 0.0f, tf = 0.0f;
    for (int i = 0; i < dim; i++) {
        float o = i == 0 ? r.o.x : (i == 1 ? r.o.y : r.o.z);
        float di = i == 0 ? r.dInv.x : (i == 1 ? r.dInv.y : r.dInv.z);
        float lo = i == 0 ? pMin.x : (i == 1 ? pMin.y : pMin.z);
        float hi = i == 0 ? pMax.x : (i == 1 ? pMax.y : pMax.z);
        float t0 = __fmul_rn(__fsub_rn(lo, o), di), t1 = __fmul_rn(__fsub_rn(hi, o), di);
        float nn = t1 < t0 ? t1 : t0, ff = t0 < t1 ? t1 : t0;
        if (i == 0) {
            tn = nn;
            tf = ff;
        } else {
            tn = tn < nn ? nn : tn;
            tf = ff < tf ? ff : tf;
        }
    }
    float tNearMax = 0.0f < tn ? tn : 0.0f, tFarMin = tf < r.tMax ? tf : r.tMax;
    if (tNearMax > tFarMin) return false;
    tMin = tNearMax;
    return true;
}

constexpr int kTopStack = 64;

// TransformedAggregate::findClosestPointFromNode (core/primitive.h:424-441), or
// the object's own traversal for an untransformed object; r2 is updated as
// the reference updates the sphere
template<int BITS, class Prim>
FCPWGB_D bool instanceClosest(int dim, const DevInstance &I, const DevObject &O, float3 c, float &r2,
                              int recordNormal, DevInteraction &cand, WideStack<kShortStack> &st,
                              uint32_t *errorWord) {
    float3 cq = c;
    float r2q = r2;
    if (I.transformed) {
        cq = xfPoint(dim, I.ti, c);
        r2q = xfR2(dim, I.ti, c, cq, r2);
    }
    uint32_t sel = kUintMax;
    NearTie<false> tie;
    Count<false> nExp, nTests;
    cand = defaultInteraction();
    bool found = wideClosest<4, BITS, Prim, false, false, kShortStack>(O.nodes, O.prims, 0u, cq, r2q, false, cand,
                                                                       sel, tie, st, errorWord, nExp, nTests);
    // the object-space radius after the walk: the winner's d*d once found
    float r2End = found ? cand.d * cand.d : r2q;
    if (found && recordNormal) cand.n = Prim::load(O.prims, sel).normal();
    if (I.transformed) {
        r2 = xfR2(dim, I.t, cq, xfPoint(dim, I.t, cq), r2End);
        if (found) xfInteraction(dim, I, c, cand);
    } else {
        r2 = r2End;
    }
    return found;
}

// TransformedAggregate::intersectFromNode (core/primitive.h:327-343)
template<int BITS, class Prim>
FCPWGB_D bool instanceRay(int dim, const DevInstance &I, const DevObject &O, DevRay &r, int occl,
                          DevInteraction &cand, WideStack<kShortStack> &st, uint32_t *errorWord) {
    DevRay rq = I.transformed ? xfRay(dim, I.ti, r) : r;
    uint32_t nExp = 0, nTests = 0;
    cand = defaultInteraction();
    bool hit = wideRay<4, BITS, Prim, kShortStack>(O.nodes, O.prims, 0u, rq, occl, cand, st, errorWord, nExp,
                                                   nTests);
    if (I.transformed) {
        r.tMax = xfRay(dim, I.t, rq).tMax;
        if (hit) xfInteraction(dim, I, r.o, cand);
    } else {
        r.tMax = rq.tMax;
    }
    return hit;
}

FCPWGB_D NodeBox topNode(const unsigned char *nodes, uint32_t i) { return loadNode<32>(nodes, i); }

// One thread per query: the top-level walk of bvh.inl:1291-1418 with aggregate
// leaves (every found candidate replaces the answer and tightens r2).
template<int BITS, class Prim>
__global__ void __launch_bounds__(kWideBlock) kInstancedClosestPoint(
    const unsigned char *__restrict__ topNodes, const uint32_t *__restrict__ topRefs, uint32_t nInstances,
    const DevInstance *__restrict__ insts, const DevObject *__restrict__ objs, const DevSphere *__restrict__ spheres,
    const uint32_t *__restrict__ perm, DevInteraction *__restrict__ out, uint32_t *__restrict__ instOut, uint32_t n,
    int dim, int recordNormal, uint32_t *errorWord) {
    __shared__ uint32_t sRef[kShortStack * kWideBlock];
    __shared__ float sD[kShortStack * kWideBlock];
    WideStack<kShortStack> st;
    st.sRef = sRef + threadIdx.x;
    st.sD = sD + threadIdx.x;
    const uint32_t q = blockIdx.x * kWideBlock + threadIdx.x;
    if (q >= n) return;
    float4 s4 = ldg4(spheres + q);
    const float3 c = make_float3(s4.x, s4.y, s4.z);
    float r2 = queryRadius2(c, s4.w);
    DevInteraction best = defaultInteraction();
    uint32_t bestInst = kUintMax;
    if (nInstances == 1) {
        DevInteraction cand;
        if (instanceClosest<BITS, Prim>(dim, insts[0], objs[insts[0].object], c, r2, recordNormal, cand, st,
                                        errorWord)) {
            best = cand;
            bestInst = 0;
        }
    } else {
        uint32_t stackNode[kTopStack];
        float stackDist[kTopStack];
        NodeBox root = topNode(topNodes, 0);
        float b0, b1;
        xboxSphere(dim, root.pMin, root.pMax, c, b0, b1);
        if (b0 <= r2) {
            r2 = fminf(r2, b1);
            stackNode[0] = 0;
            stackDist[0] = b0;
            int sp = 0;
            while (sp >= 0) {
                uint32_t ni = stackNode[sp];
                float cur = stackDist[sp];
                sp--;
                if (cur > r2) continue;
                NodeBox node = topNode(topNodes, ni);
                if (node.nPrims > 0) {
                    for (uint32_t p = 0; p < node.nPrims; p++) {
                        uint32_t k = __ldg(topRefs + node.offset + p);
                        const DevInstance &I = insts[k];
                        DevInteraction cand;
                        if (instanceClosest<BITS, Prim>(dim, I, objs[I.object], c, r2, recordNormal, cand, st,
                                                        errorWord)) {
                            r2 = fminf(r2, cand.d * cand.d);
                            best = cand;
                            bestInst = k;
                        }
                    }
                } else {
                    uint32_t li = ni + 1, ri = ni + node.offset;
                    NodeBox l = topNode(topNodes, li), rr = topNode(topNodes, ri);
                    float l0, l1, r0, r1;
                    xboxSphere(dim, l.pMin, l.pMax, c, l0, l1);
                    bool hit0 = l0 <= r2;
                    r2 = fminf(r2, l1);
                    xboxSphere(dim, rr.pMin, rr.pMax, c, r0, r1);
                    bool hit1 = r0 <= r2;
                    r2 = fminf(r2, r1);
                    if (hit0 && hit1) {
                        uint32_t closer = li, other = ri;
                        float dc = l0, dother = r0;
                        if (l0 == 0.0f && r0 == 0.0f) {
                            if (r1 < l1) { closer = ri; other = li; }
                        } else if (r0 < l0) {
                            closer = ri; other = li; dc = r0; dother = l0;
                        }
                        if (sp + 2 >= kTopStack) { atomicOr(errorWord, kErrStackOverflow); break; }
                        ++sp; stackNode[sp] = other; stackDist[sp] = dother;
                        ++sp; stackNode[sp] = closer; stackDist[sp] = dc;
                    } else if (hit0 || hit1) {
                        if (sp + 1 >= kTopStack) { atomicOr(errorWord, kErrStackOverflow); break; }
                        ++sp;
                        stackNode[sp] = hit0 ? li : ri;
                        stackDist[sp] = hit0 ? l0 : r0;
                    }
                }
            }
        }
    }
    const uint32_t slot = perm ? __ldg(perm + q) : q;
    out[slot] = best;
    if (instOut) instOut[slot] = bestInst;
}

// One thread per ray: the top-level walk of bvh.inl:655-771 with aggregate leaves.
template<int BITS, class Prim>
__global__ void __launch_bounds__(kWideBlock) kInstancedRay(
    const unsigned char *__restrict__ topNodes, const uint32_t *__restrict__ topRefs, uint32_t nInstances,
    const DevInstance *__restrict__ insts, const DevObject *__restrict__ objs, const DevRay *__restrict__ rays,
    const uint32_t *__restrict__ perm, DevInteraction *__restrict__ out, uint32_t *__restrict__ instOut, uint32_t n,
    int dim, int occl, uint32_t *errorWord) {
    __shared__ uint32_t sRef[kShortStack * kWideBlock];
    __shared__ float sD[kShortStack * kWideBlock];
    WideStack<kShortStack> st;
    st.sRef = sRef + threadIdx.x;
    st.sD = sD + threadIdx.x;
    const uint32_t q = blockIdx.x * kWideBlock + threadIdx.x;
    if (q >= n) return;
    const unsigned char *rp = reinterpret_cast<const unsigned char *>(rays + q);
    float2 a = ldg2(rp), b = ldg2(rp + 8), cc = ldg2(rp + 16), d = ldg2(rp + 24), e = ldg2(rp + 32);
    DevRay r;
    r.o = make_float3(a.x, a.y, b.x);
    r.d = make_float3(b.y, cc.x, cc.y);
    r.dInv = make_float3(d.x, d.y, e.x);
    r.tMax = e.y;
    DevInteraction best = defaultInteraction();
    uint32_t bestInst = kUintMax;
    if (nInstances == 1) {
        DevInteraction cand;
        if (instanceRay<BITS, Prim>(dim, insts[0], objs[insts[0].object], r, occl, cand, st, errorWord)) {
            best = occl ? best : cand;
            best.index = cand.index;
            bestInst = 0;
        }
    } else {
        uint32_t stackNode[kTopStack];
        float stackDist[kTopStack];
        NodeBox root = topNode(topNodes, 0);
        float t0;
        if (xboxRayCpu(dim, root.pMin, root.pMax, r, t0)) {
            stackNode[0] = 0;
            stackDist[0] = t0;
            int sp = 0;
            bool done = false;
            while (sp >= 0 && !done) {
                uint32_t ni = stackNode[sp];
                float cur = stackDist[sp];
                sp--;
                if (cur > r.tMax) continue;
                NodeBox node = topNode(topNodes, ni);
                if (node.nPrims > 0) {
                    for (uint32_t p = 0; p < node.nPrims; p++) {
                        uint32_t k = __ldg(topRefs + node.offset + p);
                        const DevInstance &I = insts[k];
                        DevInteraction cand;
                        if (instanceRay<BITS, Prim>(dim, I, objs[I.object], r, occl, cand, st, errorWord)) {
                            bestInst = k;
                            if (occl) {
                                best.index = cand.index;
                                done = true;
                                break;
                            }
                            r.tMax = fminf(r.tMax, cand.d);
                            best = cand;
                        }
                    }
                } else {
                    uint32_t li = ni + 1, ri = ni + node.offset;
                    NodeBox l = topNode(topNodes, li), rr = topNode(topNodes, ri);
                    float l0, r0;
                    bool hit0 = xboxRayCpu(dim, l.pMin, l.pMax, r, l0);
                    bool hit1 = xboxRayCpu(dim, rr.pMin, rr.pMax, r, r0);
                    if (hit0 && hit1) {
                        uint32_t closer = li, other = ri;
                        float dc = l0, dother = r0;
                        if (r0 < l0) { closer = ri; other = li; dc = r0; dother = l0; }
                        if (sp + 2 >= kTopStack) { atomicOr(errorWord, kErrStackOverflow); break; }
                        ++sp; stackNode[sp] = other; stackDist[sp] = dother;
                        ++sp; stackNode[sp] = closer; stackDist[sp] = dc;
                    } else if (hit0 || hit1) {
                        if (sp + 1 >= kTopStack) { atomicOr(errorWord, kErrStackOverflow); break; }
                        ++sp;
                        stackNode[sp] = hit0 ? li : ri;
                        stackDist[sp] = hit0 ? l0 : r0;
                    }
                }
            }
        }
    }
    const uint32_t slot = perm ? __ldg(perm + q) : q;
    out[slot] = best;
    if (instOut) instOut[slot] = bestInst;
}

}  // namespace

// ------------------------------------------------------------ scene methods
int instancedPrepare(fcpwgb_gpu_scene *s, cudaStream_t st) {
    InstancedState &I = *s->inst;
    const WideConfig &c = s->wideConfig;
    if (I.tableBits == c.bits && I.tableLeaf == c.leafSize) return FCPWGB_OK;
    I.tableBits = I.tableLeaf = -1;  // invalid until the rebuild completes
    std::vector<DevObject> table(I.objects.size());
    for (size_t k = 0; k < I.objects.size(); k++) {
        fcpwgb_gpu_scene *o = I.objects[k];
        o->wideConfig = c;
        o->wideConfig.branching = 4;
        int rc = o->ensureWide(o->stream);
        if (rc) return rc;
        table[k].nodes = (const unsigned char *)o->wideNodes.ptr;
        table[k].prims = I.dim == 3 ? (const unsigned char *)o->widePrims.ptr : (const unsigned char *)o->prims.ptr;
    }
    for (auto *o : I.objects) {
        cudaError_t e = cudaStreamSynchronize(o->stream);
        if (e != cudaSuccess) return cudaFail(e, "object wide trees");
    }
    int rc = I.objectTable.upload(table.data(), table.size() * sizeof(DevObject), st);
    if (rc) return rc;
    I.tableBits = c.bits;
    I.tableLeaf = c.leafSize;
    return FCPWGB_OK;
}

SortLimits instancedSortLimits(const InstancedState &I) {
    float ext = 1e-6f;
    for (int a = 0; a < I.dim; a++) ext = std::max(ext, I.worldBox[3 + a] - I.worldBox[a]);
    SortLimits g;
    g.lo = make_float3(I.worldBox[0] - 2.0f * ext, I.worldBox[1] - 2.0f * ext, I.worldBox[2] - 2.0f * ext);
    g.hi = make_float3(I.worldBox[3] + 2.0f * ext, I.worldBox[4] + 2.0f * ext, I.worldBox[5] + 2.0f * ext);
    g.dim = I.dim;
    return g;
}

int instancedClosest(fcpwgb_gpu_scene *s, const DevSphere *spheres, DevInteraction *out, uint32_t *instOut,
                     uint32_t n, int recordNormal, cudaStream_t st) {
    int rc = instancedPrepare(s, st);
    if (rc || n == 0) return rc;
    InstancedState &I = *s->inst;
    const uint32_t *perm = nullptr;
    const DevSphere *q = spheres;
    cudaError_t e;
    if (s->wideConfig.sortQueries && n >= 4096) {
        if ((rc = s->sortCells.ensure(sizeof(uint32_t) * kSortScratchWords))) return rc;
        if ((rc = s->sortPerm.ensure((size_t)n * sizeof(uint32_t)))) return rc;
        if ((rc = s->sortSpheres.ensure((size_t)n * sizeof(DevSphere)))) return rc;
        if ((e = launchSortQueries(instancedSortLimits(I), spheres, n, (uint32_t *)s->sortCells.ptr,
                                   (DevSphere *)s->sortSpheres.ptr, (uint32_t *)s->sortPerm.ptr, s->smCount(), st)) !=
            cudaSuccess)
            return cudaFail(e, "sort queries");
        q = (const DevSphere *)s->sortSpheres.ptr;
        perm = (const uint32_t *)s->sortPerm.ptr;
    }
    const unsigned char *tn = (const unsigned char *)I.topNodes.ptr;
    const uint32_t *tr = (const uint32_t *)I.topRefs.ptr;
    const DevInstance *ins = (const DevInstance *)I.instances.ptr;
    const DevObject *obs = (const DevObject *)I.objectTable.ptr;
    uint32_t *ew = (uint32_t *)s->errorWord.ptr;
    dim3 g((n + kWideBlock - 1) / kWideBlock), b(kWideBlock);
    const int bits = s->wideConfig.bits;
    if ((rc = s->timeStart(st))) return rc;
#define FCPWGB_INST_CP(B, P)                                                                                   \
    kInstancedClosestPoint<B, P><<<g, b, 0, st>>>(tn, tr, I.nInstances, ins, obs, q, perm, out, instOut, n,    \
                                                   I.dim, recordNormal, ew)
    if (I.dim == 3) {
        if (bits == 8) FCPWGB_INST_CP(8, Tri48Prim);
        else if (bits == 16) FCPWGB_INST_CP(16, Tri48Prim);
        else FCPWGB_INST_CP(32, Tri48Prim);
    } else {
        if (bits == 8) FCPWGB_INST_CP(8, Seg24Prim);
        else if (bits == 16) FCPWGB_INST_CP(16, Seg24Prim);
        else FCPWGB_INST_CP(32, Seg24Prim);
    }
#undef FCPWGB_INST_CP
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "instanced closest point launch");
    return s->timeEnd(st);
}

int instancedRays(fcpwgb_gpu_scene *s, const DevRay *rays, DevInteraction *out, uint32_t *instOut, uint32_t n,
                  int occl, cudaStream_t st) {
    int rc = instancedPrepare(s, st);
    if (rc || n == 0) return rc;
    InstancedState &I = *s->inst;
    const uint32_t *perm = nullptr;
    const DevRay *q = rays;
    cudaError_t e;
    if (s->wideConfig.sortQueries && n >= 4096) {
        if ((rc = s->sortCells.ensure(sizeof(uint32_t) * kSortScratchWords))) return rc;
        if ((rc = s->sortPerm.ensure((size_t)n * sizeof(uint32_t)))) return rc;
        if ((rc = s->sortRays.ensure((size_t)n * sizeof(DevRay)))) return rc;
        if ((e = launchSortRays(instancedSortLimits(I), rays, n, (uint32_t *)s->sortCells.ptr,
                                (DevRay *)s->sortRays.ptr, (uint32_t *)s->sortPerm.ptr, s->smCount(), st)) !=
            cudaSuccess)
            return cudaFail(e, "sort rays");
        q = (const DevRay *)s->sortRays.ptr;
        perm = (const uint32_t *)s->sortPerm.ptr;
    }
    const unsigned char *tn = (const unsigned char *)I.topNodes.ptr;
    const uint32_t *tr = (const uint32_t *)I.topRefs.ptr;
    const DevInstance *ins = (const DevInstance *)I.instances.ptr;
    const DevObject *obs = (const DevObject *)I.objectTable.ptr;
    uint32_t *ew = (uint32_t *)s->errorWord.ptr;
    dim3 g((n + kWideBlock - 1) / kWideBlock), b(kWideBlock);
    const int bits = s->wideConfig.bits;
    if ((rc = s->timeStart(st))) return rc;
#define FCPWGB_INST_RAY(B, P)                                                                                  \
    kInstancedRay<B, P><<<g, b, 0, st>>>(tn, tr, I.nInstances, ins, obs, q, perm, out, instOut, n, I.dim, occl, ew)
    if (I.dim == 3) {
        if (bits == 8) FCPWGB_INST_RAY(8, Tri48Prim);
        else if (bits == 16) FCPWGB_INST_RAY(16, Tri48Prim);
        else FCPWGB_INST_RAY(32, Tri48Prim);
    } else {
        if (bits == 8) FCPWGB_INST_RAY(8, Seg24Prim);
        else if (bits == 16) FCPWGB_INST_RAY(16, Seg24Prim);
        else FCPWGB_INST_RAY(32, Seg24Prim);
    }
#undef FCPWGB_INST_RAY
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "instanced ray launch");
    return s->timeEnd(st);
}

// host arrays: copies in, device call on the scene's stream, copies out, error word
int instancedHost(fcpwgb_gpu_scene *s, const void *queries, size_t queryBytes, void *out, uint32_t *instOut,
                  uint32_t n, bool rays, int flag) {
    int rc;
    size_t ob = (size_t)n * sizeof(DevInteraction);
    if ((rc = s->qIn0.ensure(queryBytes))) return rc;
    if ((rc = s->qOut.ensure(ob))) return rc;
    if (instOut && (rc = s->inst->instOut.ensure((size_t)n * sizeof(uint32_t)))) return rc;
    cudaError_t e = cudaMemcpyAsync(s->qIn0.ptr, queries, queryBytes, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    uint32_t *dInst = instOut ? (uint32_t *)s->inst->instOut.ptr : nullptr;
    rc = rays ? instancedRays(s, (const DevRay *)s->qIn0.ptr, (DevInteraction *)s->qOut.ptr, dInst, n, flag,
                              s->stream)
              : instancedClosest(s, (const DevSphere *)s->qIn0.ptr, (DevInteraction *)s->qOut.ptr, dInst, n, flag,
                                 s->stream);
    if (rc) return rc;
    uint32_t err[4] = {0, 0, 0, 0};
    if ((e = cudaMemcpyAsync(out, s->qOut.ptr, ob, cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess)
        return cudaFail(e, "cudaMemcpyAsync");
    if (instOut && (e = cudaMemcpyAsync(instOut, dInst, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                        s->stream)) != cudaSuccess)
        return cudaFail(e, "cudaMemcpyAsync");
    if ((e = cudaMemcpyAsync(err, s->errorWord.ptr, sizeof(err), cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess)
        return cudaFail(e, "cudaMemcpyAsync");
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cudaFail(e, "cudaStreamSynchronize");
    if (err[0]) {
        cudaMemsetAsync(s->errorWord.ptr, 0, sizeof(err), s->stream);
        cudaStreamSynchronize(s->stream);
        return setError(FCPWGB_ERR_TRAVERSAL, "device traversal error word " + std::to_string(err[0]));
    }
    return FCPWGB_OK;
}

}  // namespace fcpwgb

extern "C" int fcpwgb_gpu_scene_transfer_instanced(fcpwgb_gpu_scene *s, const fcpwgb_cpu_instances *inst) {
    if (!s || !inst) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    if (inst->dim != s->dim) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "instances dimension differs from the scene's");
    int rc = s->activate();
    if (rc) return rc;
    auto st = std::make_shared<InstancedState>();
    st->dim = inst->dim;
    st->nInstances = (uint32_t)inst->object.size();
    st->instObject = inst->object;
    for (size_t k = 0; k < inst->objects.size(); k++) {
        fcpwgb_gpu_scene *o = nullptr;
        if ((rc = fcpwgb_gpu_scene_create(s->dim, s->device, &o))) return rc;
        st->objects.push_back(o);
        if ((rc = fcpwgb_gpu_scene_transfer_cpu_bvh(o, inst->objects[k]))) return rc;
    }
    std::vector<DevInstance> recs(st->nInstances);
    for (uint32_t i = 0; i < st->nInstances; i++) {
        std::memcpy(recs[i].t, &inst->t[(size_t)i * 12], 48);
        std::memcpy(recs[i].ti, &inst->ti[(size_t)i * 12], 48);
        recs[i].object = inst->object[i];
        recs[i].transformed = inst->transformed[i];
        recs[i].pad0 = recs[i].pad1 = 0;
    }
    if ((rc = st->instances.upload(recs.data(), recs.size() * sizeof(DevInstance), s->stream))) return rc;
    for (int a = 0; a < 3; a++) {
        st->worldBox[a] = FLT_MAX;
        st->worldBox[3 + a] = -FLT_MAX;
    }
    for (uint32_t i = 0; i < st->nInstances; i++)
        for (int a = 0; a < 3; a++) {
            st->worldBox[a] = std::min(st->worldBox[a], inst->boxes[(size_t)i * 6 + a]);
            st->worldBox[3 + a] = std::max(st->worldBox[3 + a], inst->boxes[(size_t)i * 6 + 3 + a]);
        }
    if (inst->top) {
        st->nTopNodes = inst->top->nNodes();
        std::vector<unsigned char> nodes((size_t)st->nTopNodes * 32);
        inst->top->exportNodes(nodes.data());
        std::vector<uint32_t> refs(inst->top->primOrder().begin(), inst->top->primOrder().end());
        if (inst->top->maxDepth() > 62) return setError(FCPWGB_ERR_UNSUPPORTED, "top-level tree deeper than 62 levels");
        if ((rc = st->topNodes.upload(nodes.data(), nodes.size(), s->stream))) return rc;
        if ((rc = st->topRefs.upload(refs.data(), refs.size() * sizeof(uint32_t), s->stream))) return rc;
    } else {
        uint32_t zero = 0;
        if ((rc = st->topRefs.upload(&zero, sizeof(zero), s->stream))) return rc;
        if ((rc = st->topNodes.ensure(32))) return rc;
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cudaFail(e, "instance upload");
    s->resetTree();
    s->inst = st;
    return FCPWGB_OK;
}

static int requireInstanced(fcpwgb_gpu_scene *s) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    if (!s->inst) return setError(FCPWGB_ERR_NOT_TRANSFERRED, "no instanced scene was transferred");
    return s->activate();
}

extern "C" int fcpwgb_find_closest_points_instanced(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                    fcpwgb_interaction *out, uint32_t *instance_out, uint32_t n,
                                                    int record_normals) {
    int rc = requireInstanced(s);
    if (rc || n == 0) return rc;
    if (!spheres || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedHost(s, spheres, (size_t)n * sizeof(DevSphere), out, instance_out, n, false, record_normals);
}

extern "C" int fcpwgb_find_closest_points_instanced_device(fcpwgb_gpu_scene *s,
                                                           const fcpwgb_bounding_sphere *spheres,
                                                           fcpwgb_interaction *out, uint32_t *instance_out,
                                                           uint32_t n, int record_normals, void *stream) {
    int rc = requireInstanced(s);
    if (rc) return rc;
    if (n > 0 && (!spheres || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedClosest(s, (const DevSphere *)spheres, (DevInteraction *)out, instance_out, n, record_normals,
                            s->pick(stream));
}

extern "C" int fcpwgb_intersect_rays_instanced(fcpwgb_gpu_scene *s, const fcpwgb_ray *rays, fcpwgb_interaction *out,
                                               uint32_t *instance_out, uint32_t n, int occl) {
    int rc = requireInstanced(s);
    if (rc || n == 0) return rc;
    if (!rays || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedHost(s, rays, (size_t)n * sizeof(DevRay), out, instance_out, n, true, occl);
}

extern "C" int fcpwgb_intersect_rays_instanced_device(fcpwgb_gpu_scene *s, const fcpwgb_ray *rays,
                                                      fcpwgb_interaction *out, uint32_t *instance_out, uint32_t n,
                                                      int occl, void *stream) {
    int rc = requireInstanced(s);
    if (rc) return rc;
    if (n > 0 && (!rays || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedRays(s, (const DevRay *)rays, (DevInteraction *)out, instance_out, n, occl, s->pick(stream));
}
