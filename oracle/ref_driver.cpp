// ref_driver.cpp — TEST INFRASTRUCTURE ONLY.
//
// C entry points around the reference's own CPU Scene<DIM> (include/fcpw,
// compiled unmodified against oracle/compat/Eigen) so that tests and fixture
// generation can run the reference itself: build a scene exactly as the
// reference does, read back its flattened BVH in the GPU interop layouts
// (the same fields extractBvhNodes / extractSnchNodes / extractTriangles /
// extractLineSegments / extractSilhouetteEdges / extractSilhouetteVertices
// read, include/fcpw/gpu/bvh_interop_structures.h:172-298) and run its CPU
// queries. The private tree is reached through a partial specialisation of
// the reference's friend template CPUBvhDataExtractor (bvh.h:221-222).
#include <chrono>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace fcpw {
template<size_t A, typename B, typename C, typename D, typename E, typename F, typename G>
class CPUBvhDataExtractor;
}

#include <fcpw/fcpw.h>

struct RefTag {};

namespace fcpw {
template<size_t DIM, typename N, typename P, typename S>
class CPUBvhDataExtractor<DIM, N, P, S, RefTag, RefTag, RefTag> {
public:
    using BvhT = Bvh<DIM, N, P, S>;
    static const std::vector<N> &flat(const BvhT *b) { return b->flatTree; }
    static const std::vector<P *> &prims(const BvhT *b) { return b->primitives; }
    static const std::vector<S *> &silRefs(const BvhT *b) { return b->silhouetteRefs; }
    static int nLeafs(const BvhT *b) { return b->nLeafs; }
    static int maxDepth(const BvhT *b) { return b->maxDepth; }
};
}  // namespace fcpw

using namespace fcpw;

namespace {

struct RefScene {
    int dim = 3;
    bool snch = false;
    Scene<2> s2;
    Scene<3> s3;
};

template<size_t DIM> struct Types;
template<> struct Types<2> { using Prim = LineSegment; using Sil = SilhouetteVertex; };
template<> struct Types<3> { using Prim = Triangle; using Sil = SilhouetteEdge; };

template<size_t DIM> Scene<DIM> &sceneOf(RefScene *r);
template<> Scene<2> &sceneOf<2>(RefScene *r) { return r->s2; }
template<> Scene<3> &sceneOf<3>(RefScene *r) { return r->s3; }

void put3(float *dst, const float *src, int dim) {
    dst[0] = src[0];
    dst[1] = src[1];
    dst[2] = dim == 3 ? src[2] : 0.0f;
}

// GPUInteraction layout: p[3] n[3] uv[2] d index
template<size_t DIM> void writeInteraction(const Interaction<DIM> &i, unsigned char *out) {
    float f[10] = {0};
    for (size_t k = 0; k < DIM; k++) { f[k] = i.p[k]; f[3 + k] = i.n[k]; }
    for (size_t k = 0; k < DIM - 1; k++) f[6 + k] = i.uv[k];
    f[8] = i.d;
    uint32_t idx = i.primitiveIndex < 0 ? 0xffffffffu : (uint32_t)i.primitiveIndex;
    std::memcpy(out, f, 36);
    std::memcpy(out + 36, &idx, 4);
}

template<typename F> void parallelFor(int n, F f) {
    int nt = (int)std::thread::hardware_concurrency();
    if (nt < 1) nt = 1;
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) {
        int b = (int)((int64_t)n * t / nt), e = (int)((int64_t)n * (t + 1) / nt);
        th.emplace_back([=]() { for (int q = b; q < e; q++) f(q); });
    }
    for (auto &t : th) t.join();
}

template<size_t DIM, typename N>
int exportTree(RefScene *r, unsigned char *nodes, unsigned char *prims, unsigned char *sils, int *info) {
    using P = typename Types<DIM>::Prim;
    using S = typename std::conditional<std::is_same<N, SnchNode<DIM>>::value, typename Types<DIM>::Sil,
                                        SilhouettePrimitive<DIM>>::type;
    using X = CPUBvhDataExtractor<DIM, N, P, S, RefTag, RefTag, RefTag>;
    const Bvh<DIM, N, P, S> *b = reinterpret_cast<const Bvh<DIM, N, P, S> *>(sceneOf<DIM>(r).getSceneData()->aggregate.get());
    const auto &flat = X::flat(b);
    const auto &pr = X::prims(b);
    if (info) {
        info[0] = (int)flat.size();
        info[1] = X::nLeafs(b);
        info[2] = X::maxDepth(b);
        info[3] = (int)pr.size();
        info[4] = 0;
    }
    if (nodes) {
        size_t stride = std::is_same<N, SnchNode<DIM>>::value ? 60 : 32;
        for (size_t i = 0; i < flat.size(); i++) {
            const N &n = flat[i];
            float f[6];
            float pmin[3] = {n.box.pMin[0], n.box.pMin[1], DIM == 3 ? n.box.pMin[DIM - 1] : 0.0f};
            float pmax[3] = {n.box.pMax[0], n.box.pMax[1], DIM == 3 ? n.box.pMax[DIM - 1] : 0.0f};
            std::memcpy(f, pmin, 12);
            std::memcpy(f + 3, pmax, 12);
            unsigned char *d = nodes + i * stride;
            std::memcpy(d, f, 24);
            uint32_t np = (uint32_t)n.nReferences;
            uint32_t off = (uint32_t)(n.nReferences > 0 ? n.referenceOffset : n.secondChildOffset);
            if constexpr (std::is_same<N, SnchNode<DIM>>::value) {
                float c[5] = {n.cone.axis[0], n.cone.axis[1], DIM == 3 ? n.cone.axis[DIM - 1] : 0.0f,
                              n.cone.halfAngle, n.cone.radius};
                uint32_t ns = (uint32_t)n.nSilhouetteReferences, so = (uint32_t)n.silhouetteReferenceOffset;
                std::memcpy(d + 24, c, 20);
                std::memcpy(d + 44, &np, 4);
                std::memcpy(d + 48, &off, 4);
                std::memcpy(d + 52, &ns, 4);
                std::memcpy(d + 56, &so, 4);
            } else {
                std::memcpy(d + 24, &np, 4);
                std::memcpy(d + 28, &off, 4);
            }
        }
    }
    if (prims) {
        for (size_t k = 0; k < pr.size(); k++) {
            const P *p = pr[k];
            const auto &pos = p->soup->positions;
            if constexpr (DIM == 3) {
                float f[9];
                for (int c = 0; c < 3; c++) put3(f + 3 * c, pos[p->indices[c]].data(), 3);
                uint32_t idx = (uint32_t)p->pIndex;
                std::memcpy(prims + k * 40, f, 36);
                std::memcpy(prims + k * 40 + 36, &idx, 4);
            } else {
                float f[6];
                for (int c = 0; c < 2; c++) put3(f + 3 * c, pos[p->indices[c]].data(), 2);
                uint32_t idx = (uint32_t)p->pIndex;
                std::memcpy(prims + k * 28, f, 24);
                std::memcpy(prims + k * 28 + 24, &idx, 4);
            }
        }
    }
    if constexpr (std::is_same<N, SnchNode<DIM>>::value) {
        const auto &sr = X::silRefs(b);
        if (info) info[4] = (int)sr.size();
        if (sils) {
            for (size_t k = 0; k < sr.size(); k++) {
                const auto *s = sr[k];
                const auto &pos = s->soup->positions;
                bool f0 = s->hasFace(0), f1 = s->hasFace(1);
                Vector<DIM> n0 = f0 ? s->normal(0) : Vector<DIM>::Zero();
                Vector<DIM> n1 = f1 ? s->normal(1) : Vector<DIM>::Zero();
                uint32_t idx = (uint32_t)s->pIndex, one = (f0 && f1) ? 0u : 1u;
                if constexpr (DIM == 3) {
                    float f[12];
                    put3(f, pos[s->indices[1]].data(), 3);
                    put3(f + 3, pos[s->indices[2]].data(), 3);
                    put3(f + 6, n0.data(), 3);
                    put3(f + 9, n1.data(), 3);
                    std::memcpy(sils + k * 56, f, 48);
                    std::memcpy(sils + k * 56 + 48, &idx, 4);
                    std::memcpy(sils + k * 56 + 52, &one, 4);
                } else {
                    float f[9];
                    put3(f, pos[s->indices[1]].data(), 2);
                    put3(f + 3, n0.data(), 2);
                    put3(f + 6, n1.data(), 2);
                    std::memcpy(sils + k * 44, f, 36);
                    std::memcpy(sils + k * 44 + 36, &idx, 4);
                    std::memcpy(sils + k * 44 + 40, &one, 4);
                }
            }
        }
    }
    return 0;
}

template<size_t DIM> int exportAny(RefScene *r, unsigned char *nodes, unsigned char *prims, unsigned char *sils,
                                   int *info) {
    if (r->snch) return exportTree<DIM, SnchNode<DIM>>(r, nodes, prims, sils, info);
    return exportTree<DIM, BvhNode<DIM>>(r, nodes, prims, sils, info);
}

template<size_t DIM> Vector<DIM> vecOf(const float *p) {
    Vector<DIM> v;
    for (size_t k = 0; k < DIM; k++) v[k] = p[k];
    return v;
}

// seconds spent in f()
template<typename F> double secondsOf(F f) {
    auto t0 = std::chrono::steady_clock::now();
    f();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// the top-level Bvh of a scene of several instances, node type N (BvhNode, or SnchNode with silhouettes)
template<size_t D, typename N> int exportTop(const Aggregate<D> *agg, void *nodes, int *refs) {
    using B = Bvh<D, N, Aggregate<D>, SilhouettePrimitive<D>>;
    using X = CPUBvhDataExtractor<D, N, Aggregate<D>, SilhouettePrimitive<D>, RefTag, RefTag, RefTag>;
    const B *b = dynamic_cast<const B *>(agg);
    if (!b) return -1;
    const auto &flat = X::flat(b);
    const auto &pr = X::prims(b);
    for (size_t i = 0; nodes && i < flat.size(); i++) {
        const N &n = flat[i];
        float f[6] = {n.box.pMin[0], n.box.pMin[1], D == 3 ? n.box.pMin[D - 1] : 0.0f,
                      n.box.pMax[0], n.box.pMax[1], D == 3 ? n.box.pMax[D - 1] : 0.0f};
        unsigned char *d = (unsigned char *)nodes + i * 32;
        std::memcpy(d, f, 24);
        uint32_t np = (uint32_t)n.nReferences;
        uint32_t off = (uint32_t)(n.nReferences > 0 ? n.referenceOffset : n.secondChildOffset);
        std::memcpy(d + 24, &np, 4);
        std::memcpy(d + 28, &off, 4);
    }
    for (size_t k = 0; refs && k < pr.size(); k++) refs[k] = pr[k]->getIndex();
    return (int)flat.size();
}

}  // namespace

extern "C" {

// vectorize: Scene::build(aggregate, true), the reference's Mbvh with FCPW_SIMD_WIDTH-wide
// leaves and nodes where this file is compiled with FCPW_USE_ENOKI (without it the
// reference builds the same binary Bvh as with false, fcpw.inl:815-820,855-866)
void *ref_scene_create_ex(int dim, const float *positions, int nV, const int *indices, int nP, int aggregate,
                          int silhouettes, int vectorize) {
    RefScene *r = new RefScene;
    r->dim = dim;
    r->snch = silhouettes != 0;
    if (dim == 3) {
        std::vector<Vector3> pos(nV);
        std::vector<Vector3i> idx(nP);
        for (int i = 0; i < nV; i++) pos[i] = Vector3(positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]);
        for (int i = 0; i < nP; i++) idx[i] = Vector3i(indices[3 * i], indices[3 * i + 1], indices[3 * i + 2]);
        r->s3.setObjectCount(1);
        r->s3.setObjectVertices(pos, 0);
        r->s3.setObjectTriangles(idx, 0);
        if (r->snch) r->s3.computeSilhouettes();
        r->s3.build((AggregateType)aggregate, vectorize != 0);
    } else {
        std::vector<Vector2> pos(nV);
        std::vector<Vector2i> idx(nP);
        for (int i = 0; i < nV; i++) pos[i] = Vector2(positions[2 * i], positions[2 * i + 1]);
        for (int i = 0; i < nP; i++) idx[i] = Vector2i(indices[2 * i], indices[2 * i + 1]);
        r->s2.setObjectCount(1);
        r->s2.setObjectVertices(pos, 0);
        r->s2.setObjectLineSegments(idx, 0);
        if (r->snch) r->s2.computeSilhouettes();
        r->s2.build((AggregateType)aggregate, vectorize != 0);
    }
    return r;
}

void *ref_scene_create(int dim, const float *positions, int nV, const int *indices, int nP, int aggregate,
                       int silhouettes) {
    return ref_scene_create_ex(dim, positions, nV, indices, nP, aggregate, silhouettes, 0);
}

int ref_simd_width(void) {
#ifdef FCPW_USE_ENOKI
    return FCPW_SIMD_WIDTH;
#else
    return 0;
#endif
}

// A scene of several objects (Scene::setObjectCount, fcpw.h:29-58), each with
// its own positions and indices, and per object a list of instance
// transforms (setObjectInstanceTransforms, fcpw.h:70): nTransforms[k]
// matrices of (DIM+1)^2 row-major floats, concatenated in object order in
// transforms. An object with no transforms is one untransformed instance.
// silhouettes: Scene::computeSilhouettes before the build (every object's tree
// and the top level become SNCH trees)
void *ref_scene_create_multi_ex(int dim, int nObjects, const float *const *positions, const int *nV,
                                const int *const *indices, const int *nP, const int *nTransforms,
                                const float *transforms, int aggregate, int silhouettes) {
    RefScene *r = new RefScene;
    r->dim = dim;
    r->snch = silhouettes != 0;
    const float *tm = transforms;
    auto fill = [&](auto &scene, auto dimTag) {
        constexpr int D = (int)decltype(dimTag)::value;
        scene.setObjectCount(nObjects);
        for (int k = 0; k < nObjects; k++) {
            std::vector<Vector<D>> pos(nV[k]);
            for (int i = 0; i < nV[k]; i++) pos[i] = vecOf<D>(positions[k] + (size_t)D * i);
            scene.setObjectVertices(pos, k);
            if constexpr (D == 3) {
                std::vector<Vector3i> idx(nP[k]);
                for (int i = 0; i < nP[k]; i++)
                    idx[i] = Vector3i(indices[k][3 * i], indices[k][3 * i + 1], indices[k][3 * i + 2]);
                scene.setObjectTriangles(idx, k);
            } else {
                std::vector<Vector2i> idx(nP[k]);
                for (int i = 0; i < nP[k]; i++) idx[i] = Vector2i(indices[k][2 * i], indices[k][2 * i + 1]);
                scene.setObjectLineSegments(idx, k);
            }
            if (nTransforms[k] > 0) {
                std::vector<Transform<D>> ts;
                for (int t = 0; t < nTransforms[k]; t++) {
                    Transform<D> x;
                    for (int a = 0; a <= D; a++)
                        for (int b = 0; b <= D; b++) x.matrix()(a, b) = tm[a * (D + 1) + b];
                    tm += (D + 1) * (D + 1);
                    ts.push_back(x);
                }
                scene.setObjectInstanceTransforms(ts, k);
            }
        }
        if (r->snch) scene.computeSilhouettes();
        scene.build((AggregateType)aggregate, false);
    };
    if (dim == 3) fill(r->s3, std::integral_constant<size_t, 3>());
    else fill(r->s2, std::integral_constant<size_t, 2>());
    return r;
}

void *ref_scene_create_multi(int dim, int nObjects, const float *const *positions, const int *nV,
                             const int *const *indices, const int *nP, const int *nTransforms,
                             const float *transforms, int aggregate) {
    return ref_scene_create_multi_ex(dim, nObjects, positions, nV, indices, nP, nTransforms, transforms, aggregate,
                                     0);
}

void ref_scene_destroy(void *h) { delete (RefScene *)h; }

// info: nNodes, nLeafs, maxDepth, nPrimitives, nSilhouetteRefs
int ref_export(void *h, void *nodes, void *prims, void *sils, int *info) {
    RefScene *r = (RefScene *)h;
    if (r->dim == 3) return exportAny<3>(r, (unsigned char *)nodes, (unsigned char *)prims, (unsigned char *)sils, info);
    return exportAny<2>(r, (unsigned char *)nodes, (unsigned char *)prims, (unsigned char *)sils, info);
}

// spheres: 4 floats (c, r2) per query; out: 40 B interactions; visited may be NULL
int ref_closest_points(void *h, const float *spheres, int n, int recordNormal, void *out, int *visited) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            BoundingSphere<D> s(vecOf<D>(spheres + 4 * q), spheres[4 * q + 3]);
            Interaction<D> i;
            int nv = 0;
            agg->findClosestPointFromNode(s, i, 0, agg->getIndex(), nv, recordNormal != 0);
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
            if (visited) visited[q] = nv;
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

// The top-level Bvh of a scene of several instances (its primitives are the
// instances' aggregates): 32 B interop nodes and, per leaf reference, the
// aggregate's index (objects 0..K-1 in order, then transformed instances in
// creation order). Returns the node count, 0 when the scene has no top level.
int ref_export_top(void *h, void *nodes, int *refs) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) -> int {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        int k = exportTop<D, BvhNode<D>>(agg, nodes, refs);  // an SNCH tree when the scene has silhouettes
        if (k < 0) k = exportTop<D, SnchNode<D>>(agg, nodes, refs);
        return k < 0 ? 0 : k;
    };
    if (r->dim == 3) return run(r->s3, std::integral_constant<size_t, 3>());
    return run(r->s2, std::integral_constant<size_t, 2>());
}

// closest points and first hits on any scene, with the interaction's objectIndex
int ref_closest_points_objects(void *h, const float *spheres, int n, int recordNormal, void *out, int *object) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            BoundingSphere<D> s(vecOf<D>(spheres + 4 * q), spheres[4 * q + 3]);
            Interaction<D> i;
            int nv = 0;
            agg->findClosestPointFromNode(s, i, 0, agg->getIndex(), nv, recordNormal != 0);
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
            object[q] = i.primitiveIndex < 0 ? -1 : i.objectIndex;
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

int ref_intersect_rays_objects(void *h, const float *rays, int n, int occl, void *out, int *hit, int *object) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            const float *rr = rays + 10 * q;
            Ray<D> ray(vecOf<D>(rr), vecOf<D>(rr + 3), rr[9]);
            Interaction<D> i;
            bool hh = agg->intersect(ray, i, occl != 0);
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
            hit[q] = hh ? 1 : 0;
            object[q] = hh ? i.objectIndex : -1;
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

// rays: 40 B GPURay records (o, d, dInv, tMax); hit receives the boolean result
int ref_intersect_rays(void *h, const float *rays, int n, int occl, void *out, int *hit) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            const float *rr = rays + 10 * q;
            Ray<D> ray(vecOf<D>(rr), vecOf<D>(rr + 3), rr[9]);
            Interaction<D> i;
            bool hh = agg->intersect(ray, i, occl != 0);
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
            hit[q] = hh ? 1 : 0;
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

int ref_silhouettes(void *h, const float *spheres, const uint32_t *flip, int n, float sqMinR, float precision,
                    void *out) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            BoundingSphere<D> s(vecOf<D>(spheres + 4 * q), spheres[4 * q + 3]);
            Interaction<D> i;
            agg->findClosestSilhouettePoint(s, i, flip[q] != 0, sqMinR, precision, false);
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

// rand: 3 floats per query (the first DIM are used)
int ref_sphere_sample(void *h, const float *spheres, const float *rand, int n, void *out, int *hit) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            BoundingSphere<D> s(vecOf<D>(spheres + 4 * q), spheres[4 * q + 3]);
            Interaction<D> i;
            int hits = agg->intersect(s, i, vecOf<D>(rand + 3 * q));
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
            hit[q] = hits > 0 ? 1 : 0;
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

// updateObjectVertices (caller vertex order) followed by Scene::refit
int ref_update_and_refit(void *h, const float *positions, int nV) {
    RefScene *r = (RefScene *)h;
    if (r->dim == 3) {
        std::vector<Vector3> pos(nV);
        for (int i = 0; i < nV; i++) pos[i] = Vector3(positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]);
        r->s3.updateObjectVertices(pos, 0);
        r->s3.refit();
    } else {
        std::vector<Vector2> pos(nV);
        for (int i = 0; i < nV; i++) pos[i] = Vector2(positions[2 * i], positions[2 * i + 1]);
        r->s2.updateObjectVertices(pos, 0);
        r->s2.refit();
    }
    return 0;
}

// Scene<DIM>::contains / hasLineOfSight (fcpw.inl:1443-1460, 1501-1520): points are
// 3 floats each (the first DIM used); out receives 0 or 1
int ref_contains(void *h, const float *points, int n, uint32_t *out) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        std::vector<Vector<D>> pts(n);
        for (int q = 0; q < n; q++) pts[q] = vecOf<D>(points + 3 * q);
        std::vector<uint32_t> res;
        scene.contains(pts, res);
        for (int q = 0; q < n; q++) out[q] = res[q];
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

int ref_line_of_sight(void *h, const float *pa, const float *pb, int n, uint32_t *out) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        std::vector<Vector<D>> a(n), b(n);
        for (int q = 0; q < n; q++) {
            a[q] = vecOf<D>(pa + 3 * q);
            b[q] = vecOf<D>(pb + 3 * q);
        }
        std::vector<uint32_t> res;
        scene.hasLineOfSight(a, b, res);
        for (int q = 0; q < n; q++) out[q] = res[q];
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

// silhouettes and sphere samples on any scene, with the interaction's objectIndex
int ref_silhouettes_objects(void *h, const float *spheres, const uint32_t *flip, int n, float sqMinR,
                            float precision, void *out, int *object) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            BoundingSphere<D> s(vecOf<D>(spheres + 4 * q), spheres[4 * q + 3]);
            Interaction<D> i;
            bool found = agg->findClosestSilhouettePoint(s, i, flip[q] != 0, sqMinR, precision, false);
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
            object[q] = found ? i.objectIndex : -1;
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

int ref_sphere_sample_objects(void *h, const float *spheres, const float *rand, int n, void *out, int *hit,
                              int *object) {
    RefScene *r = (RefScene *)h;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        const Aggregate<D> *agg = scene.getSceneData()->aggregate.get();
        parallelFor(n, [&](int q) {
            BoundingSphere<D> s(vecOf<D>(spheres + 4 * q), spheres[4 * q + 3]);
            Interaction<D> i;
            int hits = agg->intersect(s, i, vecOf<D>(rand + 3 * q));
            writeInteraction<D>(i, (unsigned char *)out + 40 * (size_t)q);
            hit[q] = hits > 0 ? 1 : 0;
            object[q] = hits > 0 ? i.objectIndex : -1;
        });
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return 0;
}

// updateObjectVertices of one object (its own vertex order) followed by Scene::refit
int ref_update_object_and_refit(void *h, int object, const float *positions, int nV) {
    RefScene *r = (RefScene *)h;
    if (r->dim == 3) {
        std::vector<Vector3> pos(nV);
        for (int i = 0; i < nV; i++) pos[i] = Vector3(positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]);
        r->s3.updateObjectVertices(pos, object);
        r->s3.refit();
    } else {
        std::vector<Vector2> pos(nV);
        for (int i = 0; i < nV; i++) pos[i] = Vector2(positions[2 * i], positions[2 * i + 1]);
        r->s2.updateObjectVertices(pos, object);
        r->s2.refit();
    }
    return 0;
}

// ---- the reference's public bundled query API (Scene<DIM>::findClosestPoints,
// intersect, findClosestSilhouettePoints over std::vector, fcpw.h:172-245,
// fcpw.inl:1224-1660: one std::thread per hardware thread, contiguous query
// ranges). Each returns the seconds spent inside that one call; the records are
// converted to and from the interop layouts outside the timed span.
double ref_scene_closest_points_timed(void *h, const float *spheres, int n, void *out) {
    RefScene *r = (RefScene *)h;
    double sec = 0.0;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        std::vector<BoundingSphere<D>> q;
        q.reserve(n);
        for (int k = 0; k < n; k++) q.emplace_back(vecOf<D>(spheres + 4 * k), spheres[4 * k + 3]);
        std::vector<Interaction<D>> is;
        sec = secondsOf([&]() { scene.findClosestPoints(q, is, false); });
        for (int k = 0; k < n; k++) writeInteraction<D>(is[k], (unsigned char *)out + 40 * (size_t)k);
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return sec;
}

double ref_scene_intersect_rays_timed(void *h, const float *rays, int n, int occl, void *out) {
    RefScene *r = (RefScene *)h;
    double sec = 0.0;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        std::vector<Ray<D>> q;
        q.reserve(n);
        for (int k = 0; k < n; k++) q.emplace_back(vecOf<D>(rays + 10 * k), vecOf<D>(rays + 10 * k + 3), rays[10 * k + 9]);
        std::vector<Interaction<D>> is;
        sec = secondsOf([&]() { scene.intersect(q, is, occl != 0); });
        for (int k = 0; k < n; k++) writeInteraction<D>(is[k], (unsigned char *)out + 40 * (size_t)k);
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return sec;
}

double ref_scene_silhouettes_timed(void *h, const float *spheres, const uint32_t *flip, int n, void *out) {
    RefScene *r = (RefScene *)h;
    double sec = 0.0;
    auto run = [&](auto &scene, auto dimTag) {
        constexpr size_t D = decltype(dimTag)::value;
        std::vector<BoundingSphere<D>> q;
        q.reserve(n);
        for (int k = 0; k < n; k++) q.emplace_back(vecOf<D>(spheres + 4 * k), spheres[4 * k + 3]);
        std::vector<uint32_t> fl(flip, flip + n);
        std::vector<Interaction<D>> is;
        sec = secondsOf([&]() { scene.findClosestSilhouettePoints(q, is, fl, 0.0f, 1e-3f, false); });
        for (int k = 0; k < n; k++) writeInteraction<D>(is[k], (unsigned char *)out + 40 * (size_t)k);
    };
    if (r->dim == 3) run(r->s3, std::integral_constant<size_t, 3>());
    else run(r->s2, std::integral_constant<size_t, 2>());
    return sec;
}

}  // extern "C"
