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

#include "binary_queries.cuh"
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
    const unsigned char *nodes;     // 4-wide records
    const unsigned char *prims;     // Tri48 / Seg24 records
    const unsigned char *binNodes;  // the transferred binary tree (32 B, or 64 B SNCH records)
    const unsigned char *binPrims;  // its primitives (40 B triangles / 24 B segments)
    const unsigned char *sils;      // silhouette records of an SNCH tree, else NULL
    uint32_t maxDepth, snch;
};

struct InstancedState {
    int dim = 3;
    bool snch = false;  // every object carries a silhouette (SNCH) tree
    uint32_t nInstances = 0, nTopNodes = 0, topDepth = 0;
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
FCPWGB_D void xfInteraction(int dim, const DevInstance &I, float3 query, DevInteraction &c,
                             bool overwriteDistance = true) {
    c.p = xfPoint(dim, I.t, c.p);
    if (overwriteDistance) {
        float3 d = xsub3(c.p, query);
        c.d = __fsqrt_rn(xdot3(dim, d, d));
    }
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

// TransformedAggregate::findClosestSilhouettePointFromNode (core/primitive.h:444-466),
// or the object's own traversal for an untransformed object: the query and
// the minimum radius go to object space, the object's SNCH tree is walked
// (silhouetteBinary), the radius comes back through t and the answer is
// mapped to world space; r2 is updated as the reference updates the sphere
template<class Sil, int DIM>
FCPWGB_D bool instanceSilhouette(const DevInstance &I, const DevObject &O, float3 c, float &r2, bool flipNormal,
                                 float sqMinR, float precision, DevInteraction &cand, uint32_t *errorWord) {
    cand = defaultInteraction();
    if (!O.sils) return false;
    float3 cq = c;
    float r2q = r2, minq = sqMinR;
    if (I.transformed) {
        cq = xfPoint(DIM, I.ti, c);
        r2q = xfR2(DIM, I.ti, c, cq, r2);
        minq = xfR2(DIM, I.ti, c, cq, sqMinR);
    }
    bool found = silhouetteBinary<Sil, DIM>(O.binNodes, O.sils, cq, r2q, flipNormal, minq, precision, errorWord,
                                            cand);
    if (I.transformed) {
        r2 = xfR2(DIM, I.t, cq, xfPoint(DIM, I.t, cq), r2q);
        if (found) xfInteraction(DIM, I, c, cand);
    } else {
        r2 = r2q;
    }
    return found;
}

// TransformedAggregate::intersectFromNode for sphere sampling (core/primitive.h:392-410):
// the sphere goes to object space, the object's binary tree is sampled
// (sphereSampleBinary, rn = (u, rn1, rn2)), and the sample's point and normal
// are mapped to world space; its pdf stays the object's (applyTransform
// without overwriting the distance)
template<class Prim, int NODE_STRIDE>
FCPWGB_D bool instanceSample(int dim, const DevInstance &I, const DevObject &O, float3 c, float r2, float3 rn,
                             DevInteraction &cand, uint32_t *errorWord) {
    float3 cq = c;
    float r2q = r2;
    if (I.transformed) {
        cq = xfPoint(dim, I.ti, c);
        r2q = xfR2(dim, I.ti, c, cq, r2);
    }
    bool hit = sphereSampleBinary<Prim, NODE_STRIDE>(O.binNodes, O.binPrims, cq, r2q, rn, O.maxDepth + 1, errorWord,
                                                     cand);
    if (hit && I.transformed) xfInteraction(dim, I, c, cand, false);
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

// One thread per query: the top-level walk of bvh.inl:1435-1596 with aggregate
// leaves. The top level of a scene with silhouettes is an SNCH tree whose
// nodes keep the default cone (half angle pi: valid, always overlapping), so a
// child is entered when its box is within the radius; every silhouette found
// replaces the answer and tightens r2, and the walk stops once r2 is within
// the minimum radius.
template<class Sil, int DIM>
__global__ void __launch_bounds__(kWideBlock) kInstancedSilhouette(
    const unsigned char *__restrict__ topNodes, const uint32_t *__restrict__ topRefs, uint32_t nInstances,
    const DevInstance *__restrict__ insts, const DevObject *__restrict__ objs, const DevSphere *__restrict__ spheres,
    const uint32_t *__restrict__ flip, DevInteraction *__restrict__ out, uint32_t *__restrict__ instOut, uint32_t n,
    float sqMinR, float precision, uint32_t *errorWord) {
    const uint32_t q = blockIdx.x * kWideBlock + threadIdx.x;
    if (q >= n) return;
    float4 s4 = ldg4(spheres + q);
    const float3 c = make_float3(s4.x, s4.y, s4.z);
    float r2 = s4.w;
    const bool flipNormal = __ldg(flip + q) != 0;
    DevInteraction best = defaultInteraction();
    uint32_t bestInst = kUintMax;
    if (!(sqMinR >= r2)) {
        if (nInstances == 1) {
            DevInteraction cand;
            if (instanceSilhouette<Sil, DIM>(insts[0], objs[insts[0].object], c, r2, flipNormal, sqMinR, precision,
                                             cand, errorWord)) {
                best = cand;
                bestInst = 0;
            }
        } else {
            uint32_t stackNode[kTopStack];
            float stackDist[kTopStack];
            NodeBox root = topNode(topNodes, 0);
            float b0, b1;
            xboxSphere(DIM, root.pMin, root.pMax, c, b0, b1);
            if (b0 <= r2) {
                stackNode[0] = 0;
                stackDist[0] = b0;
                int sp = 0;
                bool done = false;
                while (sp >= 0 && !done) {
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
                            if (instanceSilhouette<Sil, DIM>(I, objs[I.object], c, r2, flipNormal, sqMinR, precision,
                                                             cand, errorWord)) {
                                r2 = fminf(r2, cand.d * cand.d);
                                best = cand;
                                bestInst = k;
                                if (sqMinR >= r2) {
                                    done = true;
                                    break;
                                }
                            }
                        }
                    } else {
                        uint32_t li = ni + 1, ri = ni + node.offset;
                        NodeBox l = topNode(topNodes, li), rr = topNode(topNodes, ri);
                        float l0, l1, r0, r1;
                        xboxSphere(DIM, l.pMin, l.pMax, c, l0, l1);
                        xboxSphere(DIM, rr.pMin, rr.pMax, c, r0, r1);
                        bool hit0 = l0 <= r2, hit1 = r0 <= r2;
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
    }
    out[q] = best;
    if (instOut) instOut[q] = bestInst;
}

// One thread per query: the stochastic top-level descent of bvh.inl:1140-1288
// with aggregate leaves: a child is chosen with probability proportional to
// its overlap weight (u = rn.x rescaled at every choice); in the leaf every
// instance is sampled with the current u (instanceSample), and one of the
// instances that hit is chosen uniformly, its sample's pdf multiplied by the
// top-level traversal pdf and divided by the number that hit.
template<class Prim, int NODE_STRIDE>
__global__ void __launch_bounds__(kWideBlock) kInstancedSphereSample(
    const unsigned char *__restrict__ topNodes, const uint32_t *__restrict__ topRefs, uint32_t nInstances,
    uint32_t topDepth, const DevInstance *__restrict__ insts, const DevObject *__restrict__ objs,
    const DevSphere *__restrict__ spheres, const float3 *__restrict__ randNums, DevInteraction *__restrict__ out,
    uint32_t *__restrict__ instOut, uint32_t n, int dim, uint32_t *errorWord) {
    const uint32_t q = blockIdx.x * kWideBlock + threadIdx.x;
    if (q >= n) return;
    float4 s4 = ldg4(spheres + q);
    const float3 c = make_float3(s4.x, s4.y, s4.z);
    const float r2 = s4.w;
    const float3 rn = randNums[q];
    DevInteraction best = defaultInteraction();
    uint32_t bestInst = kUintMax;
    if (nInstances == 1) {
        DevInteraction cand;
        if (instanceSample<Prim, NODE_STRIDE>(dim, insts[0], objs[insts[0].object], c, r2, rn, cand, errorWord)) {
            best = cand;
            bestInst = 0;
        }
    } else {
        NodeBox root = topNode(topNodes, 0);
        float b0, b1;
        xboxSphere(dim, root.pMin, root.pMax, c, b0, b1);
        if (b0 <= r2) {
            float traversalPdf = 1.0f, u = rn.x;
            uint32_t ni = 0;
            for (uint32_t step = 0; step <= topDepth; step++) {
                NodeBox node = topNode(topNodes, ni);
                if (node.nPrims > 0) {
                    float total = 0.0f;
                    for (uint32_t p = 0; p < node.nPrims; p++) {
                        uint32_t k = __ldg(topRefs + node.offset + p);
                        const DevInstance &I = insts[k];
                        DevInteraction cand;
                        if (instanceSample<Prim, NODE_STRIDE>(dim, I, objs[I.object], c, r2,
                                                              make_float3(u, rn.y, rn.z), cand, errorWord)) {
                            total += 1.0f;
                            const float prob = 1.0f / total;
                            if (u < prob) {
                                u = u / prob;
                                best = cand;
                                best.d *= traversalPdf;
                                bestInst = k;
                            } else {
                                u = (u - prob) / (1.0f - prob);
                            }
                        }
                    }
                    if (total > 0.0f) best.d /= total;
                    break;
                }
                uint32_t li = ni + 1, ri = ni + node.offset;
                NodeBox l = topNode(topNodes, li), rr = topNode(topNodes, ri);
                float l0, l1, r0, r1;
                xboxSphere(dim, l.pMin, l.pMax, c, l0, l1);
                xboxSphere(dim, rr.pMin, rr.pMax, c, r0, r1);
                const float w0 = l0 <= r2 ? 1.0f : 0.0f, w1 = r0 <= r2 ? 1.0f : 0.0f;
                const float total = w0 + w1;
                if (!(total > 0.0f)) break;
                const float p0 = w0 / total, p1 = 1.0f - p0;
                if (u < p0) {
                    u = u / p0;
                    ni = li;
                    traversalPdf *= p0;
                } else {
                    u = (u - p0) / p1;
                    ni = ri;
                    traversalPdf *= p1;
                }
                if (step == topDepth) atomicOr(errorWord, kErrStepBudget);
            }
        }
    }
    out[q] = best;
    if (instOut) instOut[q] = bestInst;
}

// Scene::refit of the top level after objects were refit (bvh.inl:548-599 over
// the instances; TransformedAggregate::boundingBox, core/primitive.h:297-300):
// every instance's box is its object's root box, or that box's corners
// mapped by t, each padded by FLT_EPSILON; a leaf's box is the union of its
// instances' boxes, an inner node's the union of its children's, nodes in
// reverse pre-order (children before parents). One thread: the top level has
// about two nodes per instance.
__global__ void kInstancedTopRefit(unsigned char *__restrict__ topNodes, const uint32_t *__restrict__ topRefs,
                                   uint32_t nTopNodes, const DevInstance *__restrict__ insts,
                                   const DevObject *__restrict__ objs, int dim) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (uint32_t ii = nTopNodes; ii-- > 0;) {
        float *f = reinterpret_cast<float *>(topNodes + (size_t)ii * 32);
        const uint32_t np = __float_as_uint(f[6]), off = __float_as_uint(f[7]);
        float lo[3] = {kFltMax, kFltMax, kFltMax}, hi[3] = {-kFltMax, -kFltMax, -kFltMax};
        if (np > 0) {
            for (uint32_t p = 0; p < np; p++) {
                const DevInstance &I = insts[topRefs[off + p]];
                const float *rb = reinterpret_cast<const float *>(objs[I.object].binNodes);
                float bl[3], bh[3];
                if (!I.transformed) {
                    for (int a = 0; a < 3; a++) {
                        bl[a] = rb[a];
                        bh[a] = rb[3 + a];
                    }
                } else {
                    for (int a = 0; a < 3; a++) {
                        bl[a] = kFltMax;
                        bh[a] = -kFltMax;
                    }
                    for (int corner = 0; corner < (1 << dim); corner++) {
                        int temp = corner;
                        float3 pc;
                        float *pp = &pc.x;
                        pc = make_float3(0.0f, 0.0f, 0.0f);
                        for (int a = 0; a < dim; a++) {
                            pp[a] = temp % 2 == 0 ? rb[a] : rb[3 + a];
                            temp /= 2;
                        }
                        float3 tq = xfPoint(dim, I.t, pc);
                        const float *qq = &tq.x;
                        for (int a = 0; a < dim; a++) {
                            const float l = __fsub_rn(qq[a], kFltEps), u = __fadd_rn(qq[a], kFltEps);
                            bl[a] = l < bl[a] ? l : bl[a];
                            bh[a] = bh[a] < u ? u : bh[a];
                        }
                    }
                    if (dim == 2) {
                        bl[2] = 0.0f;
                        bh[2] = 0.0f;
                    }
                }
                for (int a = 0; a < 3; a++) {
                    lo[a] = bl[a] < lo[a] ? bl[a] : lo[a];
                    hi[a] = hi[a] < bh[a] ? bh[a] : hi[a];
                }
            }
        } else {
            const float *lf = reinterpret_cast<const float *>(topNodes + (size_t)(ii + 1) * 32);
            const float *rf = reinterpret_cast<const float *>(topNodes + (size_t)(ii + off) * 32);
            for (int a = 0; a < 3; a++) {
                lo[a] = lf[a];
                hi[a] = lf[3 + a];
                lo[a] = rf[a] < lo[a] ? rf[a] : lo[a];
                hi[a] = hi[a] < rf[3 + a] ? rf[3 + a] : hi[a];
            }
        }
        for (int a = 0; a < 3; a++) {
            f[a] = lo[a];
            f[3 + a] = hi[a];
        }
    }
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
        table[k].binNodes = (const unsigned char *)o->nodes.ptr;
        table[k].binPrims = (const unsigned char *)o->prims.ptr;
        table[k].sils = o->snch && o->nSils > 0 ? (const unsigned char *)o->sils.ptr : nullptr;
        table[k].maxDepth = o->maxDepth;
        table[k].snch = o->snch ? 1u : 0u;
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

int instancedSilhouettes(fcpwgb_gpu_scene *s, const DevSphere *spheres, const uint32_t *flip, DevInteraction *out,
                         uint32_t *instOut, uint32_t n, float sqMinR, float precision, cudaStream_t st) {
    int rc = instancedPrepare(s, st);
    if (rc || n == 0) return rc;
    InstancedState &I = *s->inst;
    if (!I.snch) {  // no silhouette data: every result keeps its default, as for one object
        cudaError_t e = launchFillDefault(out, n, st);
        if (e == cudaSuccess && instOut) e = cudaMemsetAsync(instOut, 0xff, (size_t)n * sizeof(uint32_t), st);
        return e == cudaSuccess ? 0 : cudaFail(e, "silhouettes without silhouette data");
    }
    const unsigned char *tn = (const unsigned char *)I.topNodes.ptr;
    const uint32_t *tr = (const uint32_t *)I.topRefs.ptr;
    const DevInstance *ins = (const DevInstance *)I.instances.ptr;
    const DevObject *obs = (const DevObject *)I.objectTable.ptr;
    uint32_t *ew = (uint32_t *)s->errorWord.ptr;
    dim3 g((n + kWideBlock - 1) / kWideBlock), b(kWideBlock);
    if ((rc = s->timeStart(st))) return rc;
    if (I.dim == 3)
        kInstancedSilhouette<EdgeSil, 3><<<g, b, 0, st>>>(tn, tr, I.nInstances, ins, obs, spheres, flip, out, instOut,
                                                           n, sqMinR, precision, ew);
    else
        kInstancedSilhouette<VertexSil, 2><<<g, b, 0, st>>>(tn, tr, I.nInstances, ins, obs, spheres, flip, out,
                                                             instOut, n, sqMinR, precision, ew);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cudaFail(e, "instanced silhouette launch");
    return s->timeEnd(st);
}

int instancedSample(fcpwgb_gpu_scene *s, const DevSphere *spheres, const float3 *randNums, DevInteraction *out,
                    uint32_t *instOut, uint32_t n, cudaStream_t st) {
    int rc = instancedPrepare(s, st);
    if (rc || n == 0) return rc;
    InstancedState &I = *s->inst;
    const unsigned char *tn = (const unsigned char *)I.topNodes.ptr;
    const uint32_t *tr = (const uint32_t *)I.topRefs.ptr;
    const DevInstance *ins = (const DevInstance *)I.instances.ptr;
    const DevObject *obs = (const DevObject *)I.objectTable.ptr;
    uint32_t *ew = (uint32_t *)s->errorWord.ptr;
    dim3 g((n + kWideBlock - 1) / kWideBlock), b(kWideBlock);
    const uint32_t depth = I.topDepth + 1;
#define FCPWGB_INST_SS(P, STRIDE)                                                                              \
    kInstancedSphereSample<P, STRIDE><<<g, b, 0, st>>>(tn, tr, I.nInstances, depth, ins, obs, spheres, randNums, \
                                                       out, instOut, n, I.dim, ew)
    if (I.dim == 3) {
        if (I.snch) FCPWGB_INST_SS(TriPrim, 64);
        else FCPWGB_INST_SS(TriPrim, 32);
    } else {
        if (I.snch) FCPWGB_INST_SS(SegPrim, 64);
        else FCPWGB_INST_SS(SegPrim, 32);
    }
#undef FCPWGB_INST_SS
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cudaFail(e, "instanced sphere sampling launch");
}

// the top level after one of the objects was refit on stream st
int instancedTopRefit(fcpwgb_gpu_scene *s, cudaStream_t st) {
    int rc = instancedPrepare(s, st);
    if (rc) return rc;
    InstancedState &I = *s->inst;
    if (I.nTopNodes == 0) return FCPWGB_OK;
    kInstancedTopRefit<<<1, 1, 0, st>>>((unsigned char *)I.topNodes.ptr, (const uint32_t *)I.topRefs.ptr,
                                         I.nTopNodes, (const DevInstance *)I.instances.ptr,
                                         (const DevObject *)I.objectTable.ptr, I.dim);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cudaFail(e, "top-level refit");
}

// host arrays: copies in (queries, and for sampling the random numbers, for
// silhouettes the flip flags), device call on the scene's stream, copies out,
// error word
int instancedHostQuery(fcpwgb_gpu_scene *s, InstancedQuery kind, const void *queries, size_t queryBytes,
                       const void *second, size_t secondBytes, void *out, uint32_t *instOut, uint32_t n, int flag,
                       float sqMinR, float precision) {
    int rc;
    size_t ob = (size_t)n * sizeof(DevInteraction);
    if ((rc = s->qIn0.ensure(queryBytes))) return rc;
    if (second && (rc = s->qIn1.ensure(secondBytes))) return rc;
    if ((rc = s->qOut.ensure(ob))) return rc;
    if (instOut && (rc = s->inst->instOut.ensure((size_t)n * sizeof(uint32_t)))) return rc;
    cudaError_t e = cudaMemcpyAsync(s->qIn0.ptr, queries, queryBytes, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    if (second &&
        (e = cudaMemcpyAsync(s->qIn1.ptr, second, secondBytes, cudaMemcpyHostToDevice, s->stream)) != cudaSuccess)
        return cudaFail(e, "cudaMemcpyAsync");
    uint32_t *dInst = instOut ? (uint32_t *)s->inst->instOut.ptr : nullptr;
    DevInteraction *dOut = (DevInteraction *)s->qOut.ptr;
    switch (kind) {
        case InstancedQuery::Rays:
            rc = instancedRays(s, (const DevRay *)s->qIn0.ptr, dOut, dInst, n, flag, s->stream);
            break;
        case InstancedQuery::Sample:
            rc = instancedSample(s, (const DevSphere *)s->qIn0.ptr, (const float3 *)s->qIn1.ptr, dOut, dInst, n,
                                 s->stream);
            break;
        case InstancedQuery::Silhouette:
            rc = instancedSilhouettes(s, (const DevSphere *)s->qIn0.ptr, (const uint32_t *)s->qIn1.ptr, dOut, dInst, n,
                                      sqMinR, precision, s->stream);
            break;
        default:
            rc = instancedClosest(s, (const DevSphere *)s->qIn0.ptr, dOut, dInst, n, flag, s->stream);
    }
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

int instancedHost(fcpwgb_gpu_scene *s, const void *queries, size_t queryBytes, void *out, uint32_t *instOut,
                  uint32_t n, bool rays, int flag) {
    return instancedHostQuery(s, rays ? InstancedQuery::Rays : InstancedQuery::Closest, queries, queryBytes, nullptr,
                              0, out, instOut, n, flag, 0.0f, 0.0f);
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
    st->snch = true;
    for (auto *o : st->objects) st->snch = st->snch && o->snch;
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
        st->topDepth = inst->top->maxDepth();
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

extern "C" int fcpwgb_intersect_spheres_instanced(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                  const fcpwgb_float3 *rand_nums, fcpwgb_interaction *out,
                                                  uint32_t *instance_out, uint32_t n) {
    int rc = requireInstanced(s);
    if (rc || n == 0) return rc;
    if (!spheres || !rand_nums || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedHostQuery(s, InstancedQuery::Sample, spheres, (size_t)n * sizeof(DevSphere), rand_nums,
                              (size_t)n * sizeof(float3), out, instance_out, n, 0, 0.0f, 0.0f);
}

extern "C" int fcpwgb_intersect_spheres_instanced_device(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                         const fcpwgb_float3 *rand_nums, fcpwgb_interaction *out,
                                                         uint32_t *instance_out, uint32_t n, void *stream) {
    int rc = requireInstanced(s);
    if (rc) return rc;
    if (n > 0 && (!spheres || !rand_nums || !out))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedSample(s, (const DevSphere *)spheres, (const float3 *)rand_nums, (DevInteraction *)out,
                           instance_out, n, s->pick(stream));
}

extern "C" int fcpwgb_find_closest_silhouette_points_instanced(fcpwgb_gpu_scene *s,
                                                               const fcpwgb_bounding_sphere *spheres,
                                                               const uint32_t *flip, fcpwgb_interaction *out,
                                                               uint32_t *instance_out, uint32_t n, float sq_min_r,
                                                               float precision) {
    int rc = requireInstanced(s);
    if (rc || n == 0) return rc;
    if (!spheres || !flip || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedHostQuery(s, InstancedQuery::Silhouette, spheres, (size_t)n * sizeof(DevSphere), flip,
                              (size_t)n * sizeof(uint32_t), out, instance_out, n, 0, sq_min_r, precision);
}

extern "C" int fcpwgb_find_closest_silhouette_points_instanced_device(fcpwgb_gpu_scene *s,
                                                                      const fcpwgb_bounding_sphere *spheres,
                                                                      const uint32_t *flip, fcpwgb_interaction *out,
                                                                      uint32_t *instance_out, uint32_t n,
                                                                      float sq_min_r, float precision, void *stream) {
    int rc = requireInstanced(s);
    if (rc) return rc;
    if (n > 0 && (!spheres || !flip || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return instancedSilhouettes(s, (const DevSphere *)spheres, flip, (DevInteraction *)out, instance_out, n, sq_min_r,
                                precision, s->pick(stream));
}

static int requireObject(fcpwgb_gpu_scene *s, uint32_t object) {
    int rc = requireInstanced(s);
    if (rc) return rc;
    if (object >= s->inst->objects.size()) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "object index out of range");
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_refit_object(fcpwgb_gpu_scene *s, uint32_t object, const void *primitives,
                                             const void *silhouettes) {
    int rc = requireObject(s, object);
    if (rc) return rc;
    fcpwgb_gpu_scene *o = s->inst->objects[object];
    if ((rc = fcpwgb_gpu_scene_refit(o, primitives, silhouettes))) return rc;
    if ((rc = s->activate())) return rc;
    if ((rc = instancedTopRefit(s, s->stream))) return rc;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? FCPWGB_OK : cudaFail(e, "top-level refit");
}

extern "C" int fcpwgb_gpu_scene_update_object_vertices_device(fcpwgb_gpu_scene *s, uint32_t object,
                                                              const float *positions, uint32_t n_vertices,
                                                              void *stream) {
    int rc = requireObject(s, object);
    if (rc) return rc;
    fcpwgb_gpu_scene *o = s->inst->objects[object];
    cudaStream_t st = s->pick(stream);
    if ((rc = fcpwgb_gpu_scene_update_vertices_device(o, positions, n_vertices, st))) return rc;
    if ((rc = s->activate())) return rc;
    return instancedTopRefit(s, st);
}

extern "C" int fcpwgb_gpu_scene_export_top_nodes(fcpwgb_gpu_scene *s, void *nodes, uint32_t *n_nodes) {
    int rc = requireInstanced(s);
    if (rc) return rc;
    InstancedState &I = *s->inst;
    if (n_nodes) *n_nodes = I.nTopNodes;
    if (!nodes || I.nTopNodes == 0) return FCPWGB_OK;
    cudaError_t e = cudaMemcpyAsync(nodes, I.topNodes.ptr, (size_t)I.nTopNodes * 32, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? FCPWGB_OK : cudaFail(e, "export top-level nodes");
}
