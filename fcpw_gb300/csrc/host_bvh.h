// Host-side producer of the binary SAH BVH that the GPU query path consumes.
//
// The tree is built with the same binned-SAH recursion, split fallbacks, leaf
// rule and pre-order numbering as the reference CPU build
// (include/fcpw/aggregates/bvh.inl:40-234), so that node i here is node i of
// the reference's flatTree for the same input. Float arithmetic is written out
// in a fixed order (see vec.h) and the file is compiled without FP
// contraction, which keeps split decisions identical on x86 and Arm hosts.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "fcpw_gb300.h"
#include "vec.h"

namespace fcpwgb {

enum class Heuristic { LongestAxisCenter, SurfaceArea, OverlapSurfaceArea, Volume, OverlapVolume };

struct HostNode {
    float pMin[3], pMax[3];
    int offset;        // leaf: first reference; inner: offset to the right child
    int nReferences;   // > 0 for a leaf
    // SNCH only
    float coneAxis[3];
    float halfAngle;
    float radius;
    int silhouetteOffset;
    int nSilhouettes;
};

// One silhouette element (a 3D edge or a 2D vertex) in the reference's
// SilhouetteEdge / SilhouetteVertex index convention (silhouette_edges.inl:40-68,
// silhouette_vertices.inl:29-44).
struct HostSilhouette {
    int indices[4];    // edge: [opposite(face1), a, b, opposite(face0)]; vertex: [prev, v, next, -]
    int pIndex;
};

class HostBvh {
public:
    // Builds the tree; throws std::runtime_error on invalid input.
    HostBvh(int dim, const float *positions, uint32_t nVertices, const int32_t *indices,
            uint32_t nPrimitives, Heuristic heuristic, bool withSilhouettes, int leafSize = 4,
            int nBuckets = 8);

    int dim() const { return dim_; }
    int bvhType() const;
    bool hasSilhouettes() const { return withSilhouettes_; }
    uint32_t nNodes() const { return (uint32_t)nodes_.size(); }
    uint32_t nLeaves() const { return (uint32_t)nLeafs_; }
    uint32_t maxDepth() const { return (uint32_t)maxDepth_; }
    uint32_t nPrimitives() const { return (uint32_t)primOrder_.size(); }
    uint32_t nSilhouetteRefs() const { return (uint32_t)silRefs_.size(); }
    uint32_t nVertices() const { return (uint32_t)indexMap_.size(); }

    // interop-layout exports (reference bvh_interop_structures.h:172-298)
    void exportNodes(void *out) const;
    void exportPrimitives(void *out) const;
    void exportSilhouettes(void *out) const;
    void exportTopology(int32_t *indexMap, int32_t *primVertices, uint32_t *primIndex,
                        int32_t *silVertices) const;

    // updateObjectVertices: positions in caller vertex order
    void updatePositions(const float *positions);

    // A tree over given reference boxes (n x [pMin xyz, pMax xyz]) and
    // centroids (n x xyz): the reference's Bvh over aggregate instances
    // (fcpw.inl:1093-1101, bvh.inl:213-234). It holds no primitives;
    // primOrder() maps leaf order to the input reference index.
    static std::unique_ptr<HostBvh> fromBoxes(int dim, const float *boxes, const float *centroids, uint32_t n,
                                              Heuristic heuristic, int leafSize = 4, int nBuckets = 8);
    const std::vector<int> &primOrder() const { return primOrder_; }
    // Bvh::boundingBox (bvh.inl:615-618) and Bvh::centroid, the mean of the
    // primitive centroids in leaf order (bvh.inl:621-631)
    void rootBox(float pMin[3], float pMax[3]) const;
    void primitiveCentroidMean(float c[3]) const;

private:
    HostBvh(int dim, Heuristic heuristic, int leafSize, int nBuckets)
        : dim_(dim), heuristic_(heuristic), withSilhouettes_(false), leafSize_(leafSize), nBuckets_(nBuckets) {}
    template<int D> void buildFromBoxes(const float *boxes, const float *centroids, uint32_t n);
    template<int D> void buildAll();
    template<int D> void buildRecursive(std::vector<Box<D>> &refBoxes, std::vector<Vec<D>> &refCentroids,
                                        int parent, int start, int end, int depth);
    template<int D> float computeSplitCost(const Box<D> &l, const Box<D> &r, int nl, int nr) const;
    template<int D> void computeObjectSplit(const Box<D> &bb, const Box<D> &bc,
                                            const std::vector<Box<D>> &refBoxes,
                                            const std::vector<Vec<D>> &refCentroids,
                                            int start, int end, int &splitDim, float &splitCoord);
    template<int D> int performObjectSplit(int start, int end, int splitDim, float splitCoord,
                                           std::vector<Box<D>> &refBoxes, std::vector<Vec<D>> &refCentroids);
    void sortSoupPositions();
    void computeSilhouettesBeforeBuild();
    void assignSilhouettesAfterBuild();
    template<int D> void assignSilhouetteReferences();
    template<int D> void computeConesRecursive(const std::vector<Vec<D>> &refNormals,
                                               const std::vector<Vec<D>> &refFaceNormals,
                                               int start, int end);

    // geometry helpers in the sorted (leaf-order) vertex numbering
    template<int D> Vec<D> pos(int sortedVertex) const;
    template<int D> Vec<D> silFaceNormal(const HostSilhouette &s, int f, bool normalize) const;
    template<int D> Vec<D> silNormal(const HostSilhouette &s) const;
    template<int D> Vec<D> silCentroid(const HostSilhouette &s) const;

    int dim_;
    Heuristic heuristic_;
    bool withSilhouettes_;
    int leafSize_, nBuckets_;
    int nLeafs_ = 0, maxDepth_ = 0;

    std::vector<float> positions_;        // sorted (leaf-order) numbering, dim floats per vertex
    std::vector<int> primVerts_;          // per original primitive: corners in sorted numbering
    std::vector<int> primOrder_;          // leaf-order position -> original primitive index
    std::vector<int> indexMap_;           // caller vertex -> sorted vertex (-1 if unreferenced)
    std::vector<HostNode> nodes_;

    // silhouettes
    std::vector<int> eIndices_;           // 3 per original triangle (assignEdgeIndices)
    std::vector<HostSilhouette> silSlots_;// per edge (3D) / per vertex slot (2D), sorted numbering
    std::vector<int> silRefs_;            // silhouette references in leaf order -> slot
};

}  // namespace fcpwgb

// the object behind the C ABI's fcpwgb_cpu_bvh handle
struct fcpwgb_cpu_bvh {
    std::unique_ptr<fcpwgb::HostBvh> bvh;
};

namespace fcpwgb {
// per-node primitive count, offset and box (pMin, pMax) of the flattened binary tree
void binaryTreeArrays(const HostBvh &h, std::vector<uint32_t> &nP, std::vector<uint32_t> &off,
                      std::vector<float> &boxes);
}  // namespace fcpwgb
