// C++ drop-in for fcpw::GPUScene<DIM> (include/fcpw/fcpw_gpu.h:8-91 of the
// reference) backed by the fcpw_gb300 C ABI. Include this header instead of
// <fcpw/fcpw_gpu.h> and link libfcpw_gb300.so; the class name, constructor,
// method signatures, default arguments and the interop record types
// (float2, float3, GPURay, GPUBoundingSphere, GPUInteraction,
// FCPW_GPU_UINT_MAX; bvh_interop_structures.h:10-28,730-774) are the
// reference's, so calling code compiles unchanged. Failures throw
// std::runtime_error instead of exiting the process.
//
// transferToGPU reads the reference Bvh built by Scene<DIM>::build(...,
// vectorize=false) through the reference's friend template
// CPUBvhDataExtractor (include/fcpw/aggregates/bvh.h:221-222), flattens it in
// the interop layouts and uploads it; as in the reference only single-object
// scenes without CSG or instancing are supported, which is checked here.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace fcpw {
template<size_t A, typename B, typename C, typename D, typename E, typename F, typename G>
class CPUBvhDataExtractor;
}

#include <fcpw/fcpw.h>

#include "fcpw_gb300.h"

#ifndef FCPW_GPU_UINT_MAX
#define FCPW_GPU_UINT_MAX 4294967295
#endif

namespace fcpw {

struct alignas(8) float2 { float x, y; };
struct float3 { float x, y, z; };

struct GPURay {
    GPURay() : o{0, 0, 0}, d{0, 0, 0}, dInv{0, 0, 0}, tMax(maxFloat) {}
    GPURay(const float3 &o_, const float3 &d_, float tMax_ = maxFloat) : o(o_), d(d_), tMax(tMax_) {
        dInv.x = 1.0f / d.x;
        dInv.y = 1.0f / d.y;
        dInv.z = 1.0f / d.z;
    }
    float3 o, d, dInv;
    float tMax;
};

struct GPUBoundingSphere {
    GPUBoundingSphere() : c{0, 0, 0}, r2(0.0f) {}
    GPUBoundingSphere(const float3 &c_, float r2_) : c(c_), r2(r2_) {}
    float3 c;
    float r2;
};

struct GPUInteraction {
    GPUInteraction() : p{0, 0, 0}, n{0, 0, 0}, uv{0, 0}, d(maxFloat), index(FCPW_GPU_UINT_MAX) {}
    float3 p, n;
    float2 uv;
    float d;
    uint32_t index;
};

static_assert(sizeof(GPURay) == sizeof(fcpwgb_ray), "GPURay layout");
static_assert(sizeof(GPUBoundingSphere) == sizeof(fcpwgb_bounding_sphere), "GPUBoundingSphere layout");
static_assert(sizeof(GPUInteraction) == sizeof(fcpwgb_interaction), "GPUInteraction layout");

namespace gb300 {
struct Tag {};

inline void check(int rc) {
    if (rc != FCPWGB_OK) throw std::runtime_error(std::string("fcpw_gb300: ") + fcpwgb_last_error());
}

template<size_t DIM> inline fcpwgb_float3 f3(const Vector<DIM> &v) {
    return fcpwgb_float3{v[0], v[1], DIM == 2 ? 0.0f : v[DIM - 1]};
}
}  // namespace gb300

// read access to the reference Bvh (the friend declaration covers every specialisation)
template<size_t DIM, typename N, typename P, typename S>
class CPUBvhDataExtractor<DIM, N, P, S, gb300::Tag, gb300::Tag, gb300::Tag> {
public:
    using BvhT = Bvh<DIM, N, P, S>;
    static const std::vector<N> &flat(const BvhT *b) { return b->flatTree; }
    static const std::vector<P *> &prims(const BvhT *b) { return b->primitives; }
    static const std::vector<S *> &silRefs(const BvhT *b) { return b->silhouetteRefs; }
};

template<size_t DIM>
class GPUScene {
public:
    using Prim = typename std::conditional<DIM == 3, Triangle, LineSegment>::type;
    using Sil = typename std::conditional<DIM == 3, SilhouetteEdge, SilhouetteVertex>::type;

    GPUScene(const std::string &fcpwDirectoryPath_, bool printLogs_ = false) : printLogs(printLogs_) {
        (void)fcpwDirectoryPath_;  // kernels are precompiled; there are no shader sources to locate
        gb300::check(fcpwgb_gpu_scene_create((int)DIM, 0, &handle));
    }
    ~GPUScene() { fcpwgb_gpu_scene_destroy(handle); }
    GPUScene(const GPUScene &) = delete;
    GPUScene &operator=(const GPUScene &) = delete;

    void transferToGPU(Scene<DIM> &scene, const std::string &deviceBackend = "default") {
        if (deviceBackend != "default" && deviceBackend != "cuda")
            throw std::runtime_error("fcpw_gb300: only the CUDA backend is available");
        SceneData<DIM> *sd = scene.getSceneData();
        if (sd->soups.size() != 1 || !sd->csgTree.empty() || !sd->instanceTransforms[0].empty())
            throw std::runtime_error("fcpw_gb300: the GPU path supports single-object scenes only");
        snch = !sd->silhouetteVertexObjects.empty() || !sd->silhouetteEdgeObjects.empty();
        extract(scene, true);
        int type = DIM == 2 ? (snch ? FCPWGB_LINE_SEGMENT_SNCH : FCPWGB_LINE_SEGMENT_BVH)
                            : (snch ? FCPWGB_TRIANGLE_SNCH : FCPWGB_TRIANGLE_BVH);
        gb300::check(fcpwgb_gpu_scene_transfer(handle, type, snch ? (const void *)snchNodes.data() : bvhNodes.data(),
                                               nNodes, primBytes.data(), nPrims,
                                               silBytes.empty() ? nullptr : silBytes.data(), nSils,
                                               primVertices.data(), nVertices));
    }

    void refit(Scene<DIM> &scene, bool updateGeometry = true) {
        if (!updateGeometry) {
            gb300::check(fcpwgb_gpu_scene_refit(handle, nullptr, nullptr));
            return;
        }
        extract(scene, false);
        gb300::check(fcpwgb_gpu_scene_refit(handle, primBytes.data(), silBytes.empty() ? nullptr : silBytes.data()));
    }

    void intersect(const Eigen::MatrixXf &rayOrigins, const Eigen::MatrixXf &rayDirections,
                   const Eigen::VectorXf &rayDistanceBounds, std::vector<GPUInteraction> &interactions,
                   bool checkForOcclusion = false) {
        std::vector<GPURay> rays(rayOrigins.rows());
        for (size_t i = 0; i < rays.size(); i++) {
            float3 o{rayOrigins(i, 0), rayOrigins(i, 1), DIM == 2 ? 0.0f : rayOrigins(i, 2)};
            float3 d{rayDirections(i, 0), rayDirections(i, 1), DIM == 2 ? 0.0f : rayDirections(i, 2)};
            rays[i] = GPURay(o, d, rayDistanceBounds(i));
        }
        intersect(rays, interactions, checkForOcclusion);
    }
    void intersect(const std::vector<GPURay> &rays, std::vector<GPUInteraction> &interactions,
                   bool checkForOcclusion = false) {
        interactions.assign(rays.size(), GPUInteraction());
        gb300::check(fcpwgb_intersect_rays(handle, (const fcpwgb_ray *)rays.data(),
                                           (fcpwgb_interaction *)interactions.data(), (uint32_t)rays.size(),
                                           checkForOcclusion ? 1 : 0));
    }

    void intersect(const Eigen::MatrixXf &sphereCenters, const Eigen::VectorXf &sphereSquaredRadii,
                   const Eigen::MatrixXf &randNums, std::vector<GPUInteraction> &interactions) {
        std::vector<GPUBoundingSphere> s(sphereCenters.rows());
        std::vector<float3> r(sphereCenters.rows());
        for (size_t i = 0; i < s.size(); i++) {
            s[i] = GPUBoundingSphere(float3{sphereCenters(i, 0), sphereCenters(i, 1),
                                            DIM == 2 ? 0.0f : sphereCenters(i, 2)}, sphereSquaredRadii(i));
            r[i] = float3{randNums(i, 0), randNums(i, 1), DIM == 2 ? 0.0f : randNums(i, 2)};
        }
        intersect(s, r, interactions);
    }
    void intersect(const std::vector<GPUBoundingSphere> &boundingSpheres, const std::vector<float3> &randNums,
                   std::vector<GPUInteraction> &interactions) {
        if (randNums.size() != boundingSpheres.size()) throw std::runtime_error("fcpw_gb300: size mismatch");
        interactions.assign(boundingSpheres.size(), GPUInteraction());
        gb300::check(fcpwgb_intersect_spheres(handle, (const fcpwgb_bounding_sphere *)boundingSpheres.data(),
                                              (const fcpwgb_float3 *)randNums.data(),
                                              (fcpwgb_interaction *)interactions.data(),
                                              (uint32_t)boundingSpheres.size()));
    }

    void findClosestPoints(const Eigen::MatrixXf &queryPoints, const Eigen::VectorXf &squaredMaxRadii,
                           std::vector<GPUInteraction> &interactions, bool recordNormals = false) {
        std::vector<GPUBoundingSphere> s(queryPoints.rows());
        for (size_t i = 0; i < s.size(); i++)
            s[i] = GPUBoundingSphere(float3{queryPoints(i, 0), queryPoints(i, 1),
                                            DIM == 2 ? 0.0f : queryPoints(i, 2)}, squaredMaxRadii(i));
        findClosestPoints(s, interactions, recordNormals);
    }
    void findClosestPoints(const std::vector<GPUBoundingSphere> &boundingSpheres,
                           std::vector<GPUInteraction> &interactions, bool recordNormals = false) {
        interactions.assign(boundingSpheres.size(), GPUInteraction());
        gb300::check(fcpwgb_find_closest_points(handle, (const fcpwgb_bounding_sphere *)boundingSpheres.data(),
                                                (fcpwgb_interaction *)interactions.data(),
                                                (uint32_t)boundingSpheres.size(), recordNormals ? 1 : 0));
    }

    void findClosestSilhouettePoints(const Eigen::MatrixXf &queryPoints, const Eigen::VectorXf &squaredMaxRadii,
                                     const Eigen::VectorXi &flipNormalOrientation,
                                     std::vector<GPUInteraction> &interactions, float squaredMinRadius = 0.0f,
                                     float precision = 1e-3f) {
        std::vector<GPUBoundingSphere> s(queryPoints.rows());
        std::vector<uint32_t> flip(queryPoints.rows());
        for (size_t i = 0; i < s.size(); i++) {
            s[i] = GPUBoundingSphere(float3{queryPoints(i, 0), queryPoints(i, 1),
                                            DIM == 2 ? 0.0f : queryPoints(i, 2)}, squaredMaxRadii(i));
            flip[i] = (uint32_t)flipNormalOrientation(i);
        }
        findClosestSilhouettePoints(s, flip, interactions, squaredMinRadius, precision);
    }
    void findClosestSilhouettePoints(const std::vector<GPUBoundingSphere> &boundingSpheres,
                                     const std::vector<uint32_t> &flipNormalOrientation,
                                     std::vector<GPUInteraction> &interactions, float squaredMinRadius = 0.0f,
                                     float precision = 1e-3f) {
        if (flipNormalOrientation.size() != boundingSpheres.size())
            throw std::runtime_error("fcpw_gb300: size mismatch");
        interactions.assign(boundingSpheres.size(), GPUInteraction());
        gb300::check(fcpwgb_find_closest_silhouette_points(
            handle, (const fcpwgb_bounding_sphere *)boundingSpheres.data(), flipNormalOrientation.data(),
            (fcpwgb_interaction *)interactions.data(), (uint32_t)boundingSpheres.size(), squaredMinRadius,
            precision));
    }

    // the C ABI handle, e.g. for fcpwgb_gpu_scene_set_traversal or the device-array entry points
    fcpwgb_gpu_scene *gpuHandle() const { return handle; }

private:
    template<typename N> void extractTree(const Aggregate<DIM> *agg, bool withNodes) {
        using S = typename std::conditional<std::is_same<N, SnchNode<DIM>>::value, Sil, SilhouettePrimitive<DIM>>::type;
        using X = CPUBvhDataExtractor<DIM, N, Prim, S, gb300::Tag, gb300::Tag, gb300::Tag>;
        const Bvh<DIM, N, Prim, S> *b = dynamic_cast<const Bvh<DIM, N, Prim, S> *>(agg);
        if (!b) throw std::runtime_error("fcpw_gb300: transferToGPU needs a Scene built with a Bvh_* aggregate and "
                                         "vectorize=false");
        const auto &flat = X::flat(b);
        const auto &prims = X::prims(b);
        nNodes = (uint32_t)flat.size();
        nPrims = (uint32_t)prims.size();
        if (withNodes) {
            bvhNodes.clear();
            snchNodes.clear();
            for (const N &n : flat) {
                fcpwgb_bounding_box box{gb300::f3<DIM>(n.box.pMin), gb300::f3<DIM>(n.box.pMax)};
                uint32_t np = (uint32_t)n.nReferences;
                uint32_t off = (uint32_t)(n.nReferences > 0 ? n.referenceOffset : n.secondChildOffset);
                if constexpr (std::is_same<N, SnchNode<DIM>>::value) {
                    fcpwgb_bounding_cone cone{gb300::f3<DIM>(n.cone.axis), n.cone.halfAngle, n.cone.radius};
                    snchNodes.push_back(fcpwgb_snch_node{box, cone, np, off, (uint32_t)n.nSilhouetteReferences,
                                                         (uint32_t)n.silhouetteReferenceOffset});
                } else {
                    bvhNodes.push_back(fcpwgb_bvh_node{box, np, off});
                }
            }
        }
        // primitives in leaf order, with their corners in the caller's vertex numbering
        const PolygonSoup<DIM> &soup = *prims[0]->soup;
        std::vector<int32_t> inverse(soup.positions.size(), -1);
        for (size_t v = 0; v < soup.indexMap.size(); v++)
            if (soup.indexMap[v] >= 0) inverse[soup.indexMap[v]] = (int32_t)v;
        nVertices = (uint32_t)soup.indexMap.size();
        primBytes.clear();
        primVertices.clear();
        for (const Prim *p : prims) {
            const auto &pos = p->soup->positions;
            if constexpr (DIM == 3) {
                fcpwgb_triangle t{gb300::f3<3>(pos[p->indices[0]]), gb300::f3<3>(pos[p->indices[1]]),
                                  gb300::f3<3>(pos[p->indices[2]]), (uint32_t)p->pIndex};
                append(primBytes, t);
            } else {
                fcpwgb_line_segment s{gb300::f3<2>(pos[p->indices[0]]), gb300::f3<2>(pos[p->indices[1]]),
                                      (uint32_t)p->pIndex};
                append(primBytes, s);
            }
            for (size_t k = 0; k < DIM; k++) primVertices.push_back(inverse[p->indices[k]]);
        }
        silBytes.clear();
        nSils = 0;
        if constexpr (std::is_same<N, SnchNode<DIM>>::value) {
            const auto &refs = X::silRefs(b);
            nSils = (uint32_t)refs.size();
            for (const Sil *s : refs) {
                const auto &pos = s->soup->positions;
                bool f0 = s->hasFace(0), f1 = s->hasFace(1);
                Vector<DIM> n0 = f0 ? s->normal(0) : Vector<DIM>::Zero();
                Vector<DIM> n1 = f1 ? s->normal(1) : Vector<DIM>::Zero();
                uint32_t one = (f0 && f1) ? 0u : 1u;
                if constexpr (DIM == 3) {
                    fcpwgb_edge e{gb300::f3<3>(pos[s->indices[1]]), gb300::f3<3>(pos[s->indices[2]]),
                                  gb300::f3<3>(n0), gb300::f3<3>(n1), (uint32_t)s->pIndex, one};
                    append(silBytes, e);
                } else {
                    fcpwgb_vertex v{gb300::f3<2>(pos[s->indices[1]]), gb300::f3<2>(n0), gb300::f3<2>(n1),
                                    (uint32_t)s->pIndex, one};
                    append(silBytes, v);
                }
            }
        }
    }

    void extract(Scene<DIM> &scene, bool withNodes) {
        const Aggregate<DIM> *agg = scene.getSceneData()->aggregate.get();
        if (!agg) throw std::runtime_error("fcpw_gb300: Scene::build has not been called");
        if (snch) extractTree<SnchNode<DIM>>(agg, withNodes);
        else extractTree<BvhNode<DIM>>(agg, withNodes);
    }

    template<typename T> static void append(std::vector<unsigned char> &out, const T &rec) {
        const unsigned char *p = reinterpret_cast<const unsigned char *>(&rec);
        out.insert(out.end(), p, p + sizeof(T));
    }

    fcpwgb_gpu_scene *handle = nullptr;
    bool printLogs = false, snch = false;
    uint32_t nNodes = 0, nPrims = 0, nSils = 0, nVertices = 0;
    std::vector<fcpwgb_bvh_node> bvhNodes;
    std::vector<fcpwgb_snch_node> snchNodes;
    std::vector<unsigned char> primBytes, silBytes;
    std::vector<int32_t> primVertices;
};

}  // namespace fcpw
