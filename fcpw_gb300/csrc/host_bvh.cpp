// Host-side producer of the binary (optionally SNCH) BVH for the GPU query path.
// Build order, split rules and numbering follow the reference CPU build so the
// flattened tree is node-for-node the one the reference GPU path would upload.
#include "host_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <unordered_map>
#include <utility>

namespace fcpwgb {

namespace {
const int kMaxDepth = 64;  // FCPW_BVH_MAX_DEPTH, include/fcpw/aggregates/bvh.h:5
const float kPi = 3.14159265358979323846f;
}  // namespace

HostBvh::HostBvh(int dim, const float *positions, uint32_t nVertices, const int32_t *indices,
                 uint32_t nPrimitives, Heuristic heuristic, bool withSilhouettes, int leafSize,
                 int nBuckets)
    : dim_(dim), heuristic_(heuristic), withSilhouettes_(withSilhouettes), leafSize_(leafSize),
      nBuckets_(nBuckets) {
    if (dim != 2 && dim != 3) throw std::runtime_error("dim must be 2 or 3");
    if (nPrimitives == 0) throw std::runtime_error("cannot construct a BVH without primitives");
    if (nVertices == 0 || positions == nullptr || indices == nullptr)
        throw std::runtime_error("positions and indices are required");
    if (leafSize < 1 || nBuckets < 2) throw std::runtime_error("invalid leaf size or bucket count");

    positions_.assign(positions, positions + (size_t)nVertices * dim);
    for (size_t i = 0; i < positions_.size(); i++)
        if (!std::isfinite(positions_[i])) throw std::runtime_error("non-finite vertex position");
    primVerts_.assign(indices, indices + (size_t)nPrimitives * dim);
    for (int v : primVerts_)
        if (v < 0 || (uint32_t)v >= nVertices) throw std::runtime_error("vertex index out of range");

    // silhouettes are set up in the caller's numbering before the build
    // (Scene::computeSilhouettes, include/fcpw/fcpw.inl:429-521)
    if (withSilhouettes_) computeSilhouettesBeforeBuild();

    if (dim_ == 3) buildAll<3>(); else buildAll<2>();
}

int HostBvh::bvhType() const {
    if (dim_ == 2) return withSilhouettes_ ? FCPWGB_LINE_SEGMENT_SNCH : FCPWGB_LINE_SEGMENT_BVH;
    return withSilhouettes_ ? FCPWGB_TRIANGLE_SNCH : FCPWGB_TRIANGLE_BVH;
}

template<int D> Vec<D> HostBvh::pos(int v) const {
    Vec<D> p;
    for (int i = 0; i < D; i++) p.c[i] = positions_[(size_t)v * D + i];
    return p;
}

// ------------------------------------------------------------------ build

// SAH cost, include/fcpw/aggregates/bvh.inl:4-37 (packLeaves is off for the
// non-vectorised build the GPU path takes, fcpw.inl:812-813)
template<int D> float HostBvh::computeSplitCost(const Box<D> &l, const Box<D> &r, int nl, int nr) const {
    float cost = FLT_MAX;
    if (heuristic_ == Heuristic::SurfaceArea) {
        cost = (float)nl * l.surfaceArea() + (float)nr * r.surfaceArea();
    } else if (heuristic_ == Heuristic::OverlapSurfaceArea) {
        Box<D> bi = l.intersect(r);
        cost = ((float)nl / r.surfaceArea() + (float)nr / l.surfaceArea()) * std::fabs(bi.surfaceArea());
        if (!bi.isValid()) cost *= -1;
    } else if (heuristic_ == Heuristic::Volume) {
        cost = (float)nl * l.volume() + (float)nr * r.volume();
    } else if (heuristic_ == Heuristic::OverlapVolume) {
        Box<D> bi = l.intersect(r);
        cost = ((float)nl / r.volume() + (float)nr / l.volume()) * std::fabs(bi.volume());
        if (!bi.isValid()) cost *= -1;
    }
    return cost;
}

// binned object split, bvh.inl:40-111
template<int D>
void HostBvh::computeObjectSplit(const Box<D> &bb, const Box<D> &bc, const std::vector<Box<D>> &refBoxes,
                                 const std::vector<Vec<D>> &refCentroids, int start, int end,
                                 int &splitDim, float &splitCoord) {
    float splitCost = FLT_MAX;
    splitDim = -1;
    splitCoord = 0.0f;

    if (heuristic_ != Heuristic::LongestAxisCenter) {
        Vec<D> extent = bb.extent();
        std::vector<Box<D>> bucketBox(nBuckets_), rightBox(nBuckets_);
        std::vector<int> bucketCount(nBuckets_), rightCount(nBuckets_);

        for (int dim = 0; dim < D; dim++) {
            if (extent[dim] < 1e-6f) continue;  // flat dimension

            float bucketWidth = extent[dim] / (float)nBuckets_;
            for (int b = 0; b < nBuckets_; b++) {
                bucketBox[b] = Box<D>();
                bucketCount[b] = 0;
            }
            for (int p = start; p < end; p++) {
                int bi = (int)((refCentroids[p][dim] - bb.pMin[dim]) / bucketWidth);
                bi = std::min(std::max(bi, 0), nBuckets_ - 1);
                bucketBox[bi].expand(refBoxes[p]);
                bucketCount[bi] += 1;
            }

            // right-to-left sweep
            Box<D> boxRight;
            for (int b = nBuckets_ - 1; b > 0; b--) {
                boxRight.expand(bucketBox[b]);
                rightBox[b] = boxRight;
                rightCount[b] = bucketCount[b];
                if (b != nBuckets_ - 1) rightCount[b] += rightCount[b + 1];
            }

            // left-to-right evaluation
            Box<D> boxLeft;
            int nLeft = 0;
            for (int b = 1; b < nBuckets_; b++) {
                boxLeft.expand(bucketBox[b - 1]);
                nLeft += bucketCount[b - 1];
                if (nLeft > 0 && rightCount[b] > 0) {
                    float cost = computeSplitCost<D>(boxLeft, rightBox[b], nLeft, rightCount[b]);
                    if (cost < splitCost) {
                        splitCost = cost;
                        splitDim = dim;
                        splitCoord = bb.pMin[dim] + (float)b * bucketWidth;
                    }
                }
            }
        }
    }

    // fallback: centre of the longest centroid axis
    if (splitDim == -1) {
        splitDim = bc.maxDimension();
        splitCoord = (bc.pMin[splitDim] + bc.pMax[splitDim]) * 0.5f;
    }
}

// in-place partition with median fallback, bvh.inl:114-140
template<int D>
int HostBvh::performObjectSplit(int start, int end, int splitDim, float splitCoord,
                                std::vector<Box<D>> &refBoxes, std::vector<Vec<D>> &refCentroids) {
    int mid = start;
    for (int i = start; i < end; i++) {
        if (refCentroids[i][splitDim] < splitCoord) {
            std::swap(primOrder_[i], primOrder_[mid]);
            std::swap(refBoxes[i], refBoxes[mid]);
            std::swap(refCentroids[i], refCentroids[mid]);
            mid++;
        }
    }
    if (mid == start || mid == end) mid = start + (end - start) / 2;
    return mid;
}

// pre-order recursion, bvh.inl:143-209: left child at i + 1, right child at
// i + offset, leaf when nReferences <= leafSize or depth == MAX_DEPTH - 2
template<int D>
void HostBvh::buildRecursive(std::vector<Box<D>> &refBoxes, std::vector<Vec<D>> &refCentroids,
                             int parent, int start, int end, int depth) {
    maxDepth_ = std::max(depth, maxDepth_);
    int nodeIndex = (int)nodes_.size();
    int nRefs = end - start;

    Box<D> bb, bc;
    for (int p = start; p < end; p++) {
        bb.expand(refBoxes[p]);
        bc.expand(refCentroids[p]);
    }

    HostNode node;
    std::memset(&node, 0, sizeof(node));
    for (int i = 0; i < 3; i++) {
        node.pMin[i] = i < D ? bb.pMin[i] : 0.0f;
        node.pMax[i] = i < D ? bb.pMax[i] : 0.0f;
    }
    bool leaf = nRefs <= leafSize_ || depth == kMaxDepth - 2;
    if (leaf) {
        node.offset = start;
        node.nReferences = nRefs;
        nLeafs_++;
    } else {
        node.offset = 0;
        node.nReferences = 0;
    }
    nodes_.push_back(node);

    // the second child to arrive is the right child; it fixes the offset
    if (parent >= 0 && nodeIndex != parent + 1) nodes_[parent].offset = nodeIndex - parent;
    if (leaf) return;

    int splitDim;
    float splitCoord;
    computeObjectSplit<D>(bb, bc, refBoxes, refCentroids, start, end, splitDim, splitCoord);
    int mid = performObjectSplit<D>(start, end, splitDim, splitCoord, refBoxes, refCentroids);

    buildRecursive<D>(refBoxes, refCentroids, nodeIndex, start, mid, depth + 1);
    buildRecursive<D>(refBoxes, refCentroids, nodeIndex, mid, end, depth + 1);
}

template<int D> void HostBvh::buildAll() {
    int n = (int)primVerts_.size() / D;
    primOrder_.resize(n);
    for (int i = 0; i < n; i++) primOrder_[i] = i;

    // primitive boxes and centroids, triangles.inl:12-32, line_segments.inl
    std::vector<Box<D>> refBoxes(n);
    std::vector<Vec<D>> refCentroids(n);
    for (int i = 0; i < n; i++) {
        Vec<D> pa = pos<D>(primVerts_[(size_t)i * D + 0]);
        Vec<D> pb = pos<D>(primVerts_[(size_t)i * D + 1]);
        Box<D> b = Box<D>::fromPoint(pa);
        b.expand(pb);
        if (D == 3) {
            Vec<D> pc = pos<D>(primVerts_[(size_t)i * D + 2]);
            b.expand(pc);
            refCentroids[i] = (pa + pb + pc) / 3.0f;
        } else {
            refCentroids[i] = (pa + pb) * 0.5f;
        }
        refBoxes[i] = b;
    }

    nodes_.reserve((size_t)n * 2);
    buildRecursive<D>(refBoxes, refCentroids, -1, 0, n, 0);

    sortSoupPositions();
    if (withSilhouettes_) assignSilhouettesAfterBuild();
}

std::unique_ptr<HostBvh> HostBvh::fromBoxes(int dim, const float *boxes, const float *centroids, uint32_t n,
                                            Heuristic heuristic, int leafSize, int nBuckets) {
    if (dim != 2 && dim != 3) throw std::runtime_error("dim must be 2 or 3");
    if (n == 0) throw std::runtime_error("cannot construct a BVH without references");
    if (leafSize < 1 || nBuckets < 2) throw std::runtime_error("invalid leaf size or bucket count");
    std::unique_ptr<HostBvh> b(new HostBvh(dim, heuristic, leafSize, nBuckets));
    if (dim == 3) b->buildFromBoxes<3>(boxes, centroids, n);
    else b->buildFromBoxes<2>(boxes, centroids, n);
    return b;
}

template<int D> void HostBvh::buildFromBoxes(const float *boxes, const float *centroids, uint32_t n) {
    primOrder_.resize(n);
    for (uint32_t i = 0; i < n; i++) primOrder_[i] = (int)i;
    std::vector<Box<D>> refBoxes(n);
    std::vector<Vec<D>> refCentroids(n);
    for (uint32_t i = 0; i < n; i++) {
        for (int a = 0; a < D; a++) {
            refBoxes[i].pMin.c[a] = boxes[(size_t)i * 6 + a];
            refBoxes[i].pMax.c[a] = boxes[(size_t)i * 6 + 3 + a];
            refCentroids[i].c[a] = centroids[(size_t)i * 3 + a];
        }
    }
    nodes_.reserve((size_t)n * 2);
    buildRecursive<D>(refBoxes, refCentroids, -1, 0, (int)n, 0);
}

void HostBvh::rootBox(float pMin[3], float pMax[3]) const {
    for (int a = 0; a < 3; a++) {
        pMin[a] = nodes_.empty() ? FLT_MAX : nodes_[0].pMin[a];
        pMax[a] = nodes_.empty() ? -FLT_MAX : nodes_[0].pMax[a];
    }
}

void HostBvh::primitiveCentroidMean(float c[3]) const {
    const int D = dim_;
    float sum[3] = {0.0f, 0.0f, 0.0f};
    const size_t n = primOrder_.size();
    for (size_t k = 0; k < n; k++) {
        const int *v = &primVerts_[(size_t)primOrder_[k] * D];
        for (int a = 0; a < D; a++) {
            float x;
            if (D == 3) {  // Triangle::centroid, (pa + pb + pc) / 3
                x = ((positions_[(size_t)v[0] * D + a] + positions_[(size_t)v[1] * D + a]) +
                     positions_[(size_t)v[2] * D + a]) / 3.0f;
            } else {       // LineSegment::centroid, (pa + pb) * 0.5
                x = (positions_[(size_t)v[0] * D + a] + positions_[(size_t)v[1] * D + a]) * 0.5f;
            }
            sum[a] += x;
        }
    }
    for (int a = 0; a < 3; a++) c[a] = a < D && n > 0 ? sum[a] / (float)n : 0.0f;
}

// Renumbers vertices in leaf order, fcpw.inl:613-689.
void HostBvh::sortSoupPositions() {
    int V = (int)(positions_.size() / dim_);
    indexMap_.assign(V, -1);
    std::vector<float> sorted((size_t)V * dim_, 0.0f);
    int next = 0;
    for (const HostNode &node : nodes_) {
        for (int j = 0; j < node.nReferences; j++) {
            int prim = primOrder_[node.offset + j];
            for (int k = 0; k < dim_; k++) {
                int &v = primVerts_[(size_t)prim * dim_ + k];
                if (indexMap_[v] == -1) {
                    for (int c = 0; c < dim_; c++) sorted[(size_t)next * dim_ + c] = positions_[(size_t)v * dim_ + c];
                    indexMap_[v] = next++;
                }
                v = indexMap_[v];
            }
        }
    }
    positions_.swap(sorted);
}

void HostBvh::updatePositions(const float *positions) {
    int V = (int)indexMap_.size();
    for (int v = 0; v < V; v++) {
        int s = indexMap_[v];
        if (s < 0) continue;
        for (int c = 0; c < dim_; c++) positions_[(size_t)s * dim_ + c] = positions[(size_t)v * dim_ + c];
    }
}

// ------------------------------------------------------------ silhouettes

// Scene::computeSilhouettes, fcpw.inl:405-521 (caller numbering)
void HostBvh::computeSilhouettesBeforeBuild() {
    int n = (int)primVerts_.size() / dim_;
    if (dim_ == 3) {
        // assignEdgeIndices, fcpw.inl:405-426: edges numbered in order of first appearance
        std::map<std::pair<int, int>, int> edgeMap;
        int E = 0;
        eIndices_.resize((size_t)n * 3);
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < 3; j++) {
                int I = primVerts_[(size_t)i * 3 + j], J = primVerts_[(size_t)i * 3 + (j + 1) % 3];
                if (I > J) std::swap(I, J);
                auto it = edgeMap.find({I, J});
                if (it == edgeMap.end()) it = edgeMap.emplace(std::make_pair(I, J), E++).first;
                eIndices_[(size_t)i * 3 + j] = it->second;
            }
        }
        HostSilhouette blank = {{-1, -1, -1, -1}, -1};
        silSlots_.assign(E, blank);
        for (int i = 0; i < n; i++) {
            const int *t = &primVerts_[(size_t)i * 3];
            for (int j = 0; j < 3; j++) {
                int I = j - 1 < 0 ? 2 : j - 1, J = j, K = j + 1 > 2 ? 0 : j + 1;
                int e = eIndices_[(size_t)i * 3 + j];
                bool forward = true;
                if (t[J] > t[K]) { std::swap(J, K); forward = false; }
                HostSilhouette &s = silSlots_[e];
                s.indices[forward ? 0 : 3] = t[I];
                s.indices[1] = t[J];
                s.indices[2] = t[K];
                s.pIndex = e;
            }
        }
    } else {
        int V = (int)(positions_.size() / 2);
        HostSilhouette blank = {{-1, -1, -1, -1}, -1};
        silSlots_.assign(V, blank);
        for (int i = 0; i < n; i++) {
            int a = primVerts_[(size_t)i * 2], b = primVerts_[(size_t)i * 2 + 1];
            HostSilhouette &s1 = silSlots_[a];
            s1.indices[1] = a; s1.indices[2] = b; s1.pIndex = a;
            HostSilhouette &s2 = silSlots_[b];
            s2.indices[0] = a; s2.indices[1] = b; s2.pIndex = b;
        }
    }
}

// Post-build: remap silhouettes to the sorted numbering (fcpw.inl:709-758),
// then collect references per leaf and compute cones (bvh.inl:236-425).
void HostBvh::assignSilhouettesAfterBuild() {
    if (dim_ == 3) {
        for (HostSilhouette &s : silSlots_)
            for (int j = 0; j < 4; j++)
                if (s.indices[j] != -1) s.indices[j] = indexMap_[s.indices[j]];
        assignSilhouetteReferences<3>();
    } else {
        // slots are addressed by the new vertex number from here on
        for (int k = 0; k < (int)primOrder_.size(); k++) {
            int prim = primOrder_[k];
            int a = primVerts_[(size_t)prim * 2], b = primVerts_[(size_t)prim * 2 + 1];
            HostSilhouette &s1 = silSlots_[a];
            s1.indices[1] = a; s1.indices[2] = b; s1.pIndex = a;
            HostSilhouette &s2 = silSlots_[b];
            s2.indices[0] = a; s2.indices[1] = b; s2.pIndex = b;
        }
        assignSilhouetteReferences<2>();
    }
}

// face normal f of a silhouette, silhouette_edges.inl:45-68 / silhouette_vertices.inl:34-44
template<int D> Vec<D> HostBvh::silFaceNormal(const HostSilhouette &s, int f, bool normalize) const {
    Vec<D> n;
    if constexpr (D == 3) {
        int i = f == 0 ? 3 : 0, j = f == 0 ? 1 : 2, k = f == 0 ? 2 : 1;
        Vec<3> pa = pos<3>(s.indices[j]), pb = pos<3>(s.indices[k]), pc = pos<3>(s.indices[i]);
        n = cross(pb - pa, pc - pa);
    } else {
        int i = f == 0 ? 1 : 0;
        Vec<2> pa = pos<2>(s.indices[i]), pb = pos<2>(s.indices[i + 1]);
        Vec<2> d = pb - pa;
        n.c[0] = d.c[1];
        n.c[1] = -d.c[0];
    }
    return normalize ? normalized(n) : n;
}

static inline bool silHasFace(const HostSilhouette &s, int f, int dim) {
    if (dim == 3) return f == 0 ? s.indices[3] != -1 : s.indices[0] != -1;
    return f == 0 ? s.indices[2] != -1 : s.indices[0] != -1;
}

// normalised silhouette normal without precomputed vertex/edge normals
template<int D> Vec<D> HostBvh::silNormal(const HostSilhouette &s) const {
    Vec<D> n = Vec<D>::zero();
    if (silHasFace(s, 0, D)) n += silFaceNormal<D>(s, 0, false);
    if (silHasFace(s, 1, D)) n += silFaceNormal<D>(s, 1, false);
    return normalized(n);
}

template<int D> Vec<D> HostBvh::silCentroid(const HostSilhouette &s) const {
    if constexpr (D == 3) return (pos<3>(s.indices[1]) + pos<3>(s.indices[2])) * 0.5f;
    else return pos<2>(s.indices[1]);
}

template<int D> void HostBvh::assignSilhouetteReferences() {
    std::vector<Vec<D>> refNormals, refFaceNormals;
    silRefs_.clear();
    for (HostNode &node : nodes_) {
        std::unordered_map<int, bool> seen;
        int start = (int)silRefs_.size();
        for (int j = 0; j < node.nReferences; j++) {
            int prim = primOrder_[node.offset + j];
            for (int k = 0; k < D; k++) {
                int slot = D == 3 ? eIndices_[(size_t)prim * 3 + k] : primVerts_[(size_t)prim * 2 + k];
                if (seen.find(slot) != seen.end()) continue;
                seen[slot] = true;
                const HostSilhouette &s = silSlots_[slot];
                bool f0 = silHasFace(s, 0, D), f1 = silHasFace(s, 1, D);
                silRefs_.push_back(slot);
                refNormals.push_back(silNormal<D>(s));
                refFaceNormals.push_back(f0 ? silFaceNormal<D>(s, 0, true) : Vec<D>::zero());
                refFaceNormals.push_back(f1 ? silFaceNormal<D>(s, 1, true) : Vec<D>::zero());
            }
        }
        node.silhouetteOffset = start;
        node.nSilhouettes = (int)silRefs_.size() - start;
    }
    computeConesRecursive<D>(refNormals, refFaceNormals, 0, (int)nodes_.size());
}

// computeBoundingConesRecursive, bvh.inl:236-304
template<int D>
void HostBvh::computeConesRecursive(const std::vector<Vec<D>> &refNormals,
                                    const std::vector<Vec<D>> &refFaceNormals, int start, int end) {
    HostNode &node = nodes_[start];
    // node.cone starts as BoundingCone(): axis 0, halfAngle pi, radius 0
    for (int i = 0; i < 3; i++) node.coneAxis[i] = 0.0f;
    node.halfAngle = kPi;
    node.radius = 0.0f;

    Box<D> box;
    for (int i = 0; i < D; i++) { box.pMin.c[i] = node.pMin[i]; box.pMax.c[i] = node.pMax[i]; }
    Vec<D> centroid = box.centroid();

    Vec<D> axis = Vec<D>::zero();
    float radius = 0.0f;
    bool any = false, twoFaces = true;
    for (int i = start; i < end; i++) {
        const HostNode &child = nodes_[i];
        for (int j = 0; j < child.nSilhouettes; j++) {
            int r = child.silhouetteOffset + j;
            const HostSilhouette &s = silSlots_[silRefs_[r]];
            axis += refNormals[r];
            radius = maxf(radius, norm(silCentroid<D>(s) - centroid));
            twoFaces = twoFaces && silHasFace(s, 0, D) && silHasFace(s, 1, D);
            any = true;
        }
    }

    if (!any) {
        node.halfAngle = -kPi;
    } else if (!twoFaces) {
        node.halfAngle = kPi;
    } else {
        float axisNorm = norm(axis);
        if (axisNorm > FLT_EPSILON) {
            axis = axis / axisNorm;
            float halfAngle = 0.0f;
            for (int i = start; i < end; i++) {
                const HostNode &child = nodes_[i];
                for (int j = 0; j < child.nSilhouettes; j++) {
                    int r = child.silhouetteOffset + j;
                    for (int k = 0; k < 2; k++) {
                        float a = std::acos(maxf(-1.0f, minf(1.0f, dot(axis, refFaceNormals[2 * r + k]))));
                        halfAngle = maxf(halfAngle, a);
                    }
                }
            }
            for (int i = 0; i < 3; i++) node.coneAxis[i] = i < D ? axis.c[i] : 0.0f;
            node.halfAngle = halfAngle;
            node.radius = radius;
        }
    }

    if (node.nReferences == 0) {
        int off = node.offset;
        computeConesRecursive<D>(refNormals, refFaceNormals, start + 1, start + off);
        computeConesRecursive<D>(refNormals, refFaceNormals, start + off, end);
    }
}

// ---------------------------------------------------------------- exports

void HostBvh::exportNodes(void *out) const {
    if (!withSilhouettes_) {
        fcpwgb_bvh_node *o = (fcpwgb_bvh_node *)out;
        for (size_t i = 0; i < nodes_.size(); i++) {
            const HostNode &n = nodes_[i];
            o[i].box.pMin = {n.pMin[0], n.pMin[1], n.pMin[2]};
            o[i].box.pMax = {n.pMax[0], n.pMax[1], n.pMax[2]};
            o[i].nPrimitives = (uint32_t)n.nReferences;
            o[i].offset = (uint32_t)n.offset;
        }
    } else {
        fcpwgb_snch_node *o = (fcpwgb_snch_node *)out;
        for (size_t i = 0; i < nodes_.size(); i++) {
            const HostNode &n = nodes_[i];
            o[i].box.pMin = {n.pMin[0], n.pMin[1], n.pMin[2]};
            o[i].box.pMax = {n.pMax[0], n.pMax[1], n.pMax[2]};
            o[i].cone.axis = {n.coneAxis[0], n.coneAxis[1], n.coneAxis[2]};
            o[i].cone.halfAngle = n.halfAngle;
            o[i].cone.radius = n.radius;
            o[i].nPrimitives = (uint32_t)n.nReferences;
            o[i].offset = (uint32_t)n.offset;
            o[i].nSilhouettes = (uint32_t)n.nSilhouettes;
            o[i].silhouetteOffset = (uint32_t)n.silhouetteOffset;
        }
    }
}

void HostBvh::exportPrimitives(void *out) const {
    int n = (int)primOrder_.size();
    for (int k = 0; k < n; k++) {
        int prim = primOrder_[k];
        const int *v = &primVerts_[(size_t)prim * dim_];
        if (dim_ == 3) {
            fcpwgb_triangle &t = ((fcpwgb_triangle *)out)[k];
            Vec<3> a = pos<3>(v[0]), b = pos<3>(v[1]), c = pos<3>(v[2]);
            t.pa = {a[0], a[1], a[2]};
            t.pb = {b[0], b[1], b[2]};
            t.pc = {c[0], c[1], c[2]};
            t.index = (uint32_t)prim;
        } else {
            fcpwgb_line_segment &s = ((fcpwgb_line_segment *)out)[k];
            Vec<2> a = pos<2>(v[0]), b = pos<2>(v[1]);
            s.pa = {a[0], a[1], 0.0f};
            s.pb = {b[0], b[1], 0.0f};
            s.index = (uint32_t)prim;
        }
    }
}

// extractSilhouetteEdges / extractSilhouetteVertices, bvh_interop_structures.h:237-298
void HostBvh::exportSilhouettes(void *out) const {
    if (!withSilhouettes_) return;
    for (size_t r = 0; r < silRefs_.size(); r++) {
        const HostSilhouette &s = silSlots_[silRefs_[r]];
        bool f0 = silHasFace(s, 0, dim_), f1 = silHasFace(s, 1, dim_);
        uint32_t one = (f0 && f1) ? 0u : 1u;
        if (dim_ == 3) {
            fcpwgb_edge &e = ((fcpwgb_edge *)out)[r];
            Vec<3> a = pos<3>(s.indices[1]), b = pos<3>(s.indices[2]);
            Vec<3> n0 = f0 ? silFaceNormal<3>(s, 0, true) : Vec<3>::zero();
            Vec<3> n1 = f1 ? silFaceNormal<3>(s, 1, true) : Vec<3>::zero();
            e.pa = {a[0], a[1], a[2]};
            e.pb = {b[0], b[1], b[2]};
            e.n0 = {n0[0], n0[1], n0[2]};
            e.n1 = {n1[0], n1[1], n1[2]};
            e.index = (uint32_t)s.pIndex;
            e.hasOneAdjacentFace = one;
        } else {
            fcpwgb_vertex &v = ((fcpwgb_vertex *)out)[r];
            Vec<2> p = pos<2>(s.indices[1]);
            Vec<2> n0 = f0 ? silFaceNormal<2>(s, 0, true) : Vec<2>::zero();
            Vec<2> n1 = f1 ? silFaceNormal<2>(s, 1, true) : Vec<2>::zero();
            v.p = {p[0], p[1], 0.0f};
            v.n0 = {n0[0], n0[1], 0.0f};
            v.n1 = {n1[0], n1[1], 0.0f};
            v.index = (uint32_t)s.pIndex;
            v.hasOneAdjacentFace = one;
        }
    }
}

void HostBvh::exportTopology(int32_t *indexMap, int32_t *primVertices, uint32_t *primIndex,
                             int32_t *silVertices) const {
    // inverse map: sorted vertex -> caller vertex
    std::vector<int> inverse(indexMap_.size(), -1);
    for (size_t v = 0; v < indexMap_.size(); v++)
        if (indexMap_[v] >= 0) inverse[indexMap_[v]] = (int)v;
    if (indexMap) std::memcpy(indexMap, indexMap_.data(), indexMap_.size() * sizeof(int32_t));
    int n = (int)primOrder_.size();
    if (primVertices || primIndex) {
        for (int k = 0; k < n; k++) {
            int prim = primOrder_[k];
            if (primIndex) primIndex[k] = (uint32_t)prim;
            if (primVertices)
                for (int j = 0; j < dim_; j++)
                    primVertices[(size_t)k * dim_ + j] = inverse[primVerts_[(size_t)prim * dim_ + j]];
        }
    }
    if (silVertices && withSilhouettes_) {
        int w = dim_ + 1;
        for (size_t r = 0; r < silRefs_.size(); r++) {
            const HostSilhouette &s = silSlots_[silRefs_[r]];
            for (int j = 0; j < w; j++) {
                int v = s.indices[j];
                silVertices[r * w + j] = v < 0 ? -1 : inverse[v];
            }
        }
    }
}

}  // namespace fcpwgb
