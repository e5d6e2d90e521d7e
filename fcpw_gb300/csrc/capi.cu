// C ABI of the GB300 query path (include/fcpw_gb300.h).
//
// A fcpwgb_gpu_scene holds one transferred tree in device memory, one CUDA
// stream, the refit schedule and reusable staging buffers for the host-array
// entry points. Every tree handed in is validated on the host (offsets in
// range, a proper binary tree in pre-order, depth within the 64-entry
// traversal stack) before anything is uploaded, so device traversals never
// index outside their arrays.
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "fcpw_gb300.h"
#include "host_bvh.h"
#include "kernels.h"
#include "scene.h"

using namespace fcpwgb;

// ------------------------------------------------------------------ errors
static thread_local std::string g_lastError;

namespace fcpwgb {
int checkAligned(const void *p, size_t bytes, const char *what) {
    if (((uintptr_t)p & (uintptr_t)(bytes - 1)) == 0) return FCPWGB_OK;
    return setError(FCPWGB_ERR_INVALID_ARGUMENT,
                    std::string(what) + " array must start on a " + std::to_string(bytes) + " B boundary");
}

int setError(int code, const std::string &msg) {
    g_lastError = msg;
    return code;
}
namespace {
std::mutex gInjectMutex;
int gSkipAllocs = 0, gFailAllocs = 0;
}
bool injectedAllocFailure() {
    std::lock_guard<std::mutex> lock(gInjectMutex);
    if (gSkipAllocs > 0) {
        gSkipAllocs--;
        return false;
    }
    if (gFailAllocs > 0) {
        gFailAllocs--;
        return true;
    }
    return false;
}
int cudaFail(cudaError_t e, const char *where) {
    return setError(e == cudaErrorMemoryAllocation ? FCPWGB_ERR_OUT_OF_MEMORY : FCPWGB_ERR_CUDA,
                    std::string(where) + ": " + cudaGetErrorString(e));
}
}  // namespace fcpwgb

#define FCPWGB_CUDA(call)                                    \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cudaFail(e_, #call);   \
    } while (0)

extern "C" const char *fcpwgb_last_error(void) { return g_lastError.c_str(); }
extern "C" const char *fcpwgb_version(void) { return "fcpw_gb300 0.1 (sm_103a)"; }
extern "C" int fcpwgb_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

extern "C" int fcpwgb_debug_fail_allocations(int skip, int count) {
    if (skip < 0 || count < 0) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "negative allocation count");
    std::lock_guard<std::mutex> lock(fcpwgb::gInjectMutex);
    fcpwgb::gSkipAllocs = count > 0 ? skip : 0;
    fcpwgb::gFailAllocs = count;
    return FCPWGB_OK;
}

// ----------------------------------------------------------- CPU producer
namespace fcpwgb {
void binaryTreeArrays(const HostBvh &h, std::vector<uint32_t> &nP, std::vector<uint32_t> &off,
                      std::vector<float> &boxes) {
    uint32_t n = h.nNodes();
    bool snch = h.hasSilhouettes();
    std::vector<unsigned char> raw((size_t)n * (snch ? sizeof(fcpwgb_snch_node) : sizeof(fcpwgb_bvh_node)));
    h.exportNodes(raw.data());
    nP.resize(n);
    off.resize(n);
    boxes.resize((size_t)n * 6);
    for (uint32_t i = 0; i < n; i++) {
        const fcpwgb_bounding_box *bx;
        if (snch) {
            const fcpwgb_snch_node &nd = ((const fcpwgb_snch_node *)raw.data())[i];
            bx = &nd.box; nP[i] = nd.nPrimitives; off[i] = nd.offset;
        } else {
            const fcpwgb_bvh_node &nd = ((const fcpwgb_bvh_node *)raw.data())[i];
            bx = &nd.box; nP[i] = nd.nPrimitives; off[i] = nd.offset;
        }
        std::memcpy(&boxes[(size_t)i * 6], bx, 24);
    }
}
}  // namespace fcpwgb

extern "C" int fcpwgb_cpu_bvh_build(int dim, const float *positions, uint32_t n_vertices, const int32_t *indices,
                                    uint32_t n_primitives, int aggregate_type, int with_silhouettes,
                                    fcpwgb_cpu_bvh **out) {
    if (!out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    Heuristic h;
    switch (aggregate_type) {
        case FCPWGB_AGGREGATE_BVH_LONGEST_AXIS: h = Heuristic::LongestAxisCenter; break;
        case FCPWGB_AGGREGATE_BVH_OVERLAP_SURFACE: h = Heuristic::OverlapSurfaceArea; break;
        case FCPWGB_AGGREGATE_BVH_SURFACE_AREA: h = Heuristic::SurfaceArea; break;
        case FCPWGB_AGGREGATE_BVH_OVERLAP_VOLUME: h = Heuristic::OverlapVolume; break;
        case FCPWGB_AGGREGATE_BVH_VOLUME: h = Heuristic::Volume; break;
        default:
            return setError(FCPWGB_ERR_UNSUPPORTED,
                            "the GPU path needs a BVH aggregate (Bvh_*); Baseline is not supported");
    }
    try {
        auto *b = new fcpwgb_cpu_bvh;
        b->bvh.reset(new HostBvh(dim, positions, n_vertices, indices, n_primitives, h, with_silhouettes != 0));
        *out = b;
    } catch (const std::bad_alloc &) {
        return setError(FCPWGB_ERR_OUT_OF_MEMORY, "host allocation failed while building the BVH");
    } catch (const std::exception &e) {
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, e.what());
    }
    return FCPWGB_OK;
}

extern "C" void fcpwgb_cpu_bvh_destroy(fcpwgb_cpu_bvh *bvh) { delete bvh; }

extern "C" int fcpwgb_cpu_bvh_info(const fcpwgb_cpu_bvh *b, fcpwgb_bvh_info *info) {
    if (!b || !info) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    info->dim = b->bvh->dim();
    info->bvh_type = b->bvh->bvhType();
    info->n_nodes = b->bvh->nNodes();
    info->n_leaves = b->bvh->nLeaves();
    info->max_depth = b->bvh->maxDepth();
    info->n_primitives = b->bvh->nPrimitives();
    info->n_silhouettes = b->bvh->nSilhouetteRefs();
    info->n_vertices = b->bvh->nVertices();
    return FCPWGB_OK;
}

extern "C" int fcpwgb_cpu_bvh_export(const fcpwgb_cpu_bvh *b, void *nodes, void *primitives, void *silhouettes) {
    if (!b) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL bvh");
    if (nodes) b->bvh->exportNodes(nodes);
    if (primitives) b->bvh->exportPrimitives(primitives);
    if (silhouettes) b->bvh->exportSilhouettes(silhouettes);
    return FCPWGB_OK;
}

extern "C" int fcpwgb_cpu_bvh_export_topology(const fcpwgb_cpu_bvh *b, int32_t *index_map, int32_t *prim_vertices,
                                              uint32_t *prim_index, int32_t *sil_vertices) {
    if (!b) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL bvh");
    b->bvh->exportTopology(index_map, prim_vertices, prim_index, sil_vertices);
    return FCPWGB_OK;
}

extern "C" int fcpwgb_cpu_bvh_export_wide(const fcpwgb_cpu_bvh *b, int branching, int bits, int leaf_size,
                                          void *nodes, int32_t *child_binary, uint32_t *n_nodes,
                                          uint32_t *node_bytes) {
    if (!b || !n_nodes || !node_bytes) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<uint32_t> nP, off;
    std::vector<float> boxes;
    binaryTreeArrays(*b->bvh, nP, off, boxes);
    WideHost w;
    if (!(branching == 2 || branching == 4 || branching == 8) || !(bits == 8 || bits == 16 || bits == 32))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "branching must be 2/4/8 and bits 8/16/32");
    if (leaf_size < 0 || leaf_size > 15) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "leaf_size must be 0..15");
    if (!buildWideTree(branching, bits, nP, off, boxes, w, leaf_size))
        return setError(FCPWGB_ERR_UNSUPPORTED, "this tree cannot be collapsed into the requested wide layout");
    *n_nodes = w.nNodes;
    *node_bytes = (uint32_t)wideNodeBytes(branching, bits);
    if (nodes) std::memcpy(nodes, w.nodes.data(), w.nodes.size());
    if (child_binary) std::memcpy(child_binary, w.childBinary.data(), w.childBinary.size() * sizeof(int32_t));
    return FCPWGB_OK;
}

extern "C" int fcpwgb_cpu_bvh_update_positions(fcpwgb_cpu_bvh *b, const float *positions) {
    if (!b || !positions) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    b->bvh->updatePositions(positions);
    return FCPWGB_OK;
}

// ------------------------------------------------------------- GPU scene
namespace fcpwgb {

int GpuScene::activate() const {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cudaFail(e, "cudaSetDevice");
    return FCPWGB_OK;
}

SceneView GpuScene::view() const {
    SceneView v;
    v.dim = dim;
    v.snch = snch;
    v.nodes = (const unsigned char *)nodes.ptr;
    v.prims = (const unsigned char *)prims.ptr;
    v.sils = (const unsigned char *)sils.ptr;
    v.nNodes = nNodes;
    v.nPrims = nPrims;
    v.nSils = nSils;
    v.maxDepth = maxDepth;
    v.errorWord = (uint32_t *)errorWord.ptr;
    return v;
}

// device entry points run on the stream they are given; NULL is the CUDA default stream
cudaStream_t GpuScene::pick(void *s) const { return (cudaStream_t)s; }

}  // namespace fcpwgb

static size_t primBytes(int dim) { return dim == 3 ? sizeof(DevTriangle) : sizeof(DevSegment2); }
static size_t silBytes(int dim) { return dim == 3 ? sizeof(DevEdge) : sizeof(DevVertex2); }

extern "C" int fcpwgb_gpu_scene_create(int dim, int device, fcpwgb_gpu_scene **out) {
    if (!out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (dim != 2 && dim != 3) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
    int count = fcpwgb_device_count();
    if (count == 0) return setError(FCPWGB_ERR_CUDA, "no CUDA device is visible");
    if (device < 0 || device >= count) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "device index out of range");
    std::unique_ptr<fcpwgb_gpu_scene> s(new fcpwgb_gpu_scene);
    s->dim = dim;
    s->device = device;
    FCPWGB_CUDA(cudaSetDevice(device));
    FCPWGB_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    int rc = s->errorWord.ensure(sizeof(uint32_t) * 4);
    if (rc) return rc;
    FCPWGB_CUDA(cudaMemsetAsync(s->errorWord.ptr, 0, sizeof(uint32_t) * 4, s->stream));
    FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
    *out = s.release();
    return FCPWGB_OK;
}

extern "C" void fcpwgb_gpu_scene_destroy(fcpwgb_gpu_scene *s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) {
        cudaStreamSynchronize(s->stream);
        cudaStreamDestroy(s->stream);
    }
    delete s;
}

// Validates a pre-order binary tree; fills parents, leaves and the max depth.
static int validateTree(const std::vector<uint32_t> &nPrims, const std::vector<uint32_t> &offsets,
                        uint32_t nPrimitives, std::vector<int32_t> &parents, std::vector<uint32_t> &leaves,
                        uint32_t &maxDepth) {
    uint32_t n = (uint32_t)nPrims.size();
    parents.assign(n, -2);
    leaves.clear();
    maxDepth = 0;
    std::vector<std::pair<uint32_t, uint32_t>> stack;  // (node, depth)
    stack.push_back({0u, 0u});
    parents[0] = -1;
    uint32_t visited = 0;
    uint64_t primsCovered = 0;
    while (!stack.empty()) {
        auto [i, depth] = stack.back();
        stack.pop_back();
        visited++;
        if (depth > 62) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "tree deeper than 62 levels");
        maxDepth = depth > maxDepth ? depth : maxDepth;
        if (nPrims[i] > 0) {
            if ((uint64_t)offsets[i] + nPrims[i] > nPrimitives)
                return setError(FCPWGB_ERR_INVALID_ARGUMENT, "leaf primitive range out of bounds");
            primsCovered += nPrims[i];
            leaves.push_back(i);
        } else {
            uint64_t l = (uint64_t)i + 1, r = (uint64_t)i + offsets[i];
            if (offsets[i] < 2 || r >= n || l >= n)
                return setError(FCPWGB_ERR_INVALID_ARGUMENT, "inner node child offset out of range");
            if (parents[l] != -2 || parents[r] != -2)
                return setError(FCPWGB_ERR_INVALID_ARGUMENT, "node referenced by two parents");
            parents[l] = (int32_t)i;
            parents[r] = (int32_t)i;
            stack.push_back({(uint32_t)r, depth + 1});
            stack.push_back({(uint32_t)l, depth + 1});
        }
    }
    if (visited != n) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "unreachable nodes in the tree");
    (void)primsCovered;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_transfer(fcpwgb_gpu_scene *s, int bvh_type, const void *nodes, uint32_t n_nodes,
                                         const void *primitives, uint32_t n_primitives, const void *silhouettes,
                                         uint32_t n_silhouettes, const int32_t *prim_vertices,
                                         uint32_t n_vertices) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    int rc = s->activate();
    if (rc) return rc;
    bool is2d = bvh_type == FCPWGB_LINE_SEGMENT_BVH || bvh_type == FCPWGB_LINE_SEGMENT_SNCH;
    bool is3d = bvh_type == FCPWGB_TRIANGLE_BVH || bvh_type == FCPWGB_TRIANGLE_SNCH;
    if (!is2d && !is3d) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "unknown bvh_type");
    if ((is2d && s->dim != 2) || (is3d && s->dim != 3))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "bvh_type does not match the scene dimension");
    bool snch = bvh_type == FCPWGB_LINE_SEGMENT_SNCH || bvh_type == FCPWGB_TRIANGLE_SNCH;
    if (!nodes || n_nodes == 0 || !primitives || n_primitives == 0)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "a non-empty tree and primitive array are required");
    if (snch && n_silhouettes > 0 && !silhouettes)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "silhouettes missing");

    // gather node topology and check it
    std::vector<uint32_t> nP(n_nodes), off(n_nodes);
    std::vector<uint32_t> nS, sOff;
    if (snch) { nS.resize(n_nodes); sOff.resize(n_nodes); }
    for (uint32_t i = 0; i < n_nodes; i++) {
        if (snch) {
            const fcpwgb_snch_node &nd = ((const fcpwgb_snch_node *)nodes)[i];
            nP[i] = nd.nPrimitives; off[i] = nd.offset; nS[i] = nd.nSilhouettes; sOff[i] = nd.silhouetteOffset;
            if ((uint64_t)nd.silhouetteOffset + nd.nSilhouettes > n_silhouettes)
                return setError(FCPWGB_ERR_INVALID_ARGUMENT, "silhouette range out of bounds");
        } else {
            const fcpwgb_bvh_node &nd = ((const fcpwgb_bvh_node *)nodes)[i];
            nP[i] = nd.nPrimitives; off[i] = nd.offset;
        }
    }
    std::vector<int32_t> parents;
    std::vector<uint32_t> leaves;
    uint32_t maxDepth = 0;
    rc = validateTree(nP, off, n_primitives, parents, leaves, maxDepth);
    if (rc) return rc;
    if (prim_vertices) {
        for (uint64_t k = 0; k < (uint64_t)n_primitives * s->dim; k++)
            if (prim_vertices[k] < 0 || (uint32_t)prim_vertices[k] >= n_vertices)
                return setError(FCPWGB_ERR_INVALID_ARGUMENT, "prim_vertices index out of range");
    }

    // device layouts
    std::vector<unsigned char> hNodes((size_t)n_nodes * (snch ? 64 : 32), 0);
    for (uint32_t i = 0; i < n_nodes; i++) {
        unsigned char *d = hNodes.data() + (size_t)i * (snch ? 64 : 32);
        if (snch) {
            const fcpwgb_snch_node &nd = ((const fcpwgb_snch_node *)nodes)[i];
            std::memcpy(d, &nd.box, 24);
            std::memcpy(d + 24, &nd.nPrimitives, 4);
            std::memcpy(d + 28, &nd.offset, 4);
            std::memcpy(d + 32, &nd.cone, 20);
            std::memcpy(d + 52, &nd.nSilhouettes, 4);
            std::memcpy(d + 56, &nd.silhouetteOffset, 4);
        } else {
            std::memcpy(d, (const unsigned char *)nodes + (size_t)i * 32, 32);
        }
    }
    std::vector<unsigned char> hPrims((size_t)n_primitives * primBytes(s->dim), 0);
    if (s->dim == 3) {
        std::memcpy(hPrims.data(), primitives, hPrims.size());
    } else {
        for (uint32_t k = 0; k < n_primitives; k++) {
            const fcpwgb_line_segment &sg = ((const fcpwgb_line_segment *)primitives)[k];
            DevSegment2 d;
            d.pa = make_float2(sg.pa.x, sg.pa.y);
            d.pb = make_float2(sg.pb.x, sg.pb.y);
            d.index = sg.index;
            d.pad = 0;
            std::memcpy(hPrims.data() + (size_t)k * sizeof(DevSegment2), &d, sizeof(d));
        }
    }
    std::vector<unsigned char> hSils;
    if (snch && n_silhouettes > 0) {
        hSils.resize((size_t)n_silhouettes * silBytes(s->dim));
        if (s->dim == 3) {
            std::memcpy(hSils.data(), silhouettes, hSils.size());
        } else {
            for (uint32_t k = 0; k < n_silhouettes; k++) {
                const fcpwgb_vertex &v = ((const fcpwgb_vertex *)silhouettes)[k];
                DevVertex2 d;
                d.p = make_float2(v.p.x, v.p.y);
                d.n0 = make_float2(v.n0.x, v.n0.y);
                d.n1 = make_float2(v.n1.x, v.n1.y);
                d.index = v.index;
                d.hasOneAdjacentFace = v.hasOneAdjacentFace;
                std::memcpy(hSils.data() + (size_t)k * sizeof(DevVertex2), &d, sizeof(d));
            }
        }
    }

    // upload
    s->resetTree();
    if ((rc = s->nodes.upload(hNodes.data(), hNodes.size(), s->stream))) return rc;
    if ((rc = s->prims.upload(hPrims.data(), hPrims.size(), s->stream))) return rc;
    if (!hSils.empty() && (rc = s->sils.upload(hSils.data(), hSils.size(), s->stream))) return rc;
    if ((rc = s->parents.upload(parents.data(), parents.size() * sizeof(int32_t), s->stream))) return rc;
    if ((rc = s->leaves.upload(leaves.data(), leaves.size() * sizeof(uint32_t), s->stream))) return rc;
    if ((rc = s->counters.ensure((size_t)n_nodes * sizeof(uint32_t)))) return rc;
    std::vector<int32_t> origVerts;
    std::vector<uint32_t> csrOff, csrCorner;
    if (prim_vertices) {
        if ((rc = s->primVerts.upload(prim_vertices, (size_t)n_primitives * s->dim * sizeof(int32_t), s->stream)))
            return rc;
        s->nVertices = n_vertices;
        // corner table in original primitive order and the vertex -> corner CSR
        // (corners of a vertex listed in increasing corner id: a fixed order)
        int d = s->dim;
        origVerts.assign((size_t)n_primitives * d, -1);
        for (uint32_t k = 0; k < n_primitives; k++) {
            uint32_t idx = d == 3 ? ((const fcpwgb_triangle *)primitives)[k].index
                                  : ((const fcpwgb_line_segment *)primitives)[k].index;
            if (idx >= n_primitives) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "primitive index out of range");
            for (int j = 0; j < d; j++) origVerts[(size_t)idx * d + j] = prim_vertices[(size_t)k * d + j];
        }
        csrOff.assign((size_t)n_vertices + 1, 0);
        for (int32_t v : origVerts) {
            if (v < 0) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "primitive indices are not a permutation");
            csrOff[(size_t)v + 1]++;
        }
        for (uint32_t v = 0; v < n_vertices; v++) csrOff[v + 1] += csrOff[v];
        csrCorner.resize(origVerts.size());
        std::vector<uint32_t> cursor(csrOff.begin(), csrOff.end() - 1);
        for (uint32_t c = 0; c < (uint32_t)origVerts.size(); c++) csrCorner[cursor[origVerts[c]]++] = c;
        if ((rc = s->origVerts.upload(origVerts.data(), origVerts.size() * sizeof(int32_t), s->stream))) return rc;
        if ((rc = s->csrOff.upload(csrOff.data(), csrOff.size() * sizeof(uint32_t), s->stream))) return rc;
        if ((rc = s->csrCorner.upload(csrCorner.data(), csrCorner.size() * sizeof(uint32_t), s->stream))) return rc;
    }
    FCPWGB_CUDA(cudaStreamSynchronize(s->stream));

    s->bvhType = bvh_type;
    s->snch = snch;
    s->nNodes = n_nodes;
    s->nPrims = n_primitives;
    s->nSils = snch ? n_silhouettes : 0;
    s->nLeaves = (uint32_t)leaves.size();
    s->maxDepth = maxDepth;
    s->hasTopology = prim_vertices != nullptr;
    if (!s->hasTopology) s->nVertices = 0;
    s->hostNP = nP;
    s->hostOff = off;
    s->hostBoxes.resize((size_t)n_nodes * 6);
    for (uint32_t i = 0; i < n_nodes; i++)
        std::memcpy(&s->hostBoxes[(size_t)i * 6], hNodes.data() + (size_t)i * (snch ? 64 : 32), 24);
    std::memcpy(s->rootBox, s->hostBoxes.data(), 24);
    s->transferred = true;
    s->treeVersion++;
    resolveStaticScratch(s);
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_transfer_cpu_bvh(fcpwgb_gpu_scene *s, const fcpwgb_cpu_bvh *b) {
    if (!s || !b) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    const HostBvh &h = *b->bvh;
    bool snch = h.hasSilhouettes();
    std::vector<unsigned char> nodes((size_t)h.nNodes() * (snch ? sizeof(fcpwgb_snch_node) : sizeof(fcpwgb_bvh_node)));
    std::vector<unsigned char> prims((size_t)h.nPrimitives() * (h.dim() == 3 ? sizeof(fcpwgb_triangle) : sizeof(fcpwgb_line_segment)));
    std::vector<unsigned char> sils((size_t)h.nSilhouetteRefs() * (h.dim() == 3 ? sizeof(fcpwgb_edge) : sizeof(fcpwgb_vertex)));
    std::vector<int32_t> primVerts((size_t)h.nPrimitives() * h.dim());
    std::vector<int32_t> silVerts((size_t)h.nSilhouetteRefs() * (h.dim() + 1));
    h.exportNodes(nodes.data());
    h.exportPrimitives(prims.data());
    if (snch) h.exportSilhouettes(sils.data());
    h.exportTopology(nullptr, primVerts.data(), nullptr, snch ? silVerts.data() : nullptr);
    int rc = fcpwgb_gpu_scene_transfer(s, h.bvhType(), nodes.data(), h.nNodes(), prims.data(), h.nPrimitives(),
                                       sils.empty() ? nullptr : sils.data(), h.nSilhouetteRefs(), primVerts.data(),
                                       h.nVertices());
    if (rc) return rc;
    if (snch && !silVerts.empty()) {
        if ((rc = s->silVerts.upload(silVerts.data(), silVerts.size() * sizeof(int32_t), s->stream))) return rc;
        FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
    }
    return FCPWGB_OK;
}

// ------------------------------------------------------------------ GPU build
// Builds the tree on the device (k_build.cu), reads the interop arrays back
// and hands them to the validating transfer, so the scene is set up exactly
// as for a host-built tree.
// sahHeuristic >= 0: the reference's binned SAH build with that heuristic
// (k_sah_build.cu) instead of the linear BVH
static int gpuBuild(fcpwgb_gpu_scene *s, const float *positions, uint32_t nVertices, const int32_t *indices,
                    uint32_t nPrims, uint32_t maxLeaf, cudaStream_t st, int sahHeuristic = -1) {
    const int dim = s->dim;
    if (!positions || !indices || nPrims == 0 || nVertices == 0)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "non-empty positions and indices are required");
    if (sahHeuristic < 0 && (maxLeaf == 0 || maxLeaf > 15))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "max_leaf_size must be 1..15");
    if (nPrims >= (1u << 27)) return setError(FCPWGB_ERR_UNSUPPORTED, "too many primitives for the GPU build");
    const size_t recBytes = dim == 3 ? sizeof(fcpwgb_triangle) : sizeof(fcpwgb_line_segment);
    DeviceBuffer scratch, nodes, prims, verts, counters;
    int rc;
    if ((rc = scratch.ensure(lbvhScratchWords(nPrims) * sizeof(uint32_t)))) return rc;
    if ((rc = nodes.ensure((2 * (size_t)nPrims) * sizeof(fcpwgb_bvh_node)))) return rc;
    if ((rc = prims.ensure((size_t)nPrims * recBytes))) return rc;
    if ((rc = verts.ensure((size_t)nPrims * dim * sizeof(int32_t)))) return rc;
    if ((rc = counters.ensure(16 * sizeof(uint32_t)))) return rc;
    uint32_t *cnt = (uint32_t *)counters.ptr;
    uint32_t host[16] = {0};
    FCPWGB_CUDA(launchCheckIndices(indices, (size_t)nPrims * dim, nVertices, cnt + 8, s->smCount(), st));
    FCPWGB_CUDA(cudaMemcpyAsync(host + 8, cnt + 8, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    FCPWGB_CUDA(cudaStreamSynchronize(st));
    if (host[8]) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "vertex index out of range");
    FCPWGB_CUDA(cudaMemsetAsync(cnt + 9, 0, sizeof(uint32_t), st));
    if (sahHeuristic >= 0) {
        DeviceBuffer sNodes, sPrims, sVerts;
        uint32_t nNodes = 0;
        if ((rc = buildSahTree(dim, sahHeuristic, positions, indices, nPrims, cnt + 9, st, sNodes, sPrims, sVerts,
                               nNodes)))
            return rc;
        FCPWGB_CUDA(cudaMemcpyAsync(host, cnt, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        FCPWGB_CUDA(cudaStreamSynchronize(st));
        if (host[9]) return setError(FCPWGB_ERR_TRAVERSAL, "GPU build: a subtree stack overflowed");
        std::vector<unsigned char> hN((size_t)nNodes * sizeof(fcpwgb_bvh_node)), hP((size_t)nPrims * recBytes);
        std::vector<int32_t> hV((size_t)nPrims * dim);
        FCPWGB_CUDA(cudaMemcpyAsync(hN.data(), sNodes.ptr, hN.size(), cudaMemcpyDeviceToHost, st));
        FCPWGB_CUDA(cudaMemcpyAsync(hP.data(), sPrims.ptr, hP.size(), cudaMemcpyDeviceToHost, st));
        FCPWGB_CUDA(cudaMemcpyAsync(hV.data(), sVerts.ptr, hV.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        FCPWGB_CUDA(cudaStreamSynchronize(st));
        return fcpwgb_gpu_scene_transfer(s, dim == 3 ? FCPWGB_TRIANGLE_BVH : FCPWGB_LINE_SEGMENT_BVH, hN.data(),
                                         nNodes, hP.data(), nPrims, nullptr, 0, hV.data(), nVertices);
    }
    FCPWGB_CUDA(launchBuildLbvh(positions, indices, dim, nPrims, maxLeaf, (uint32_t *)scratch.ptr,
                                (unsigned char *)nodes.ptr, (unsigned char *)prims.ptr, (int32_t *)verts.ptr, cnt,
                                cnt + 9, s->smCount(), st));
    FCPWGB_CUDA(cudaMemcpyAsync(host, cnt, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    FCPWGB_CUDA(cudaStreamSynchronize(st));
    if (host[9]) return setError(FCPWGB_ERR_TRAVERSAL, "GPU build: a bottom-up pass ran past its step bound");
    const uint32_t nLeaves = host[0];
    if (nLeaves == 0 || nLeaves > nPrims) return setError(FCPWGB_ERR_TRAVERSAL, "GPU build: bad leaf count");
    const uint32_t nNodes = 2 * nLeaves - 1;
    std::vector<unsigned char> hNodes((size_t)nNodes * sizeof(fcpwgb_bvh_node)), hPrims((size_t)nPrims * recBytes);
    std::vector<int32_t> hVerts((size_t)nPrims * dim);
    FCPWGB_CUDA(cudaMemcpyAsync(hNodes.data(), nodes.ptr, hNodes.size(), cudaMemcpyDeviceToHost, st));
    FCPWGB_CUDA(cudaMemcpyAsync(hPrims.data(), prims.ptr, hPrims.size(), cudaMemcpyDeviceToHost, st));
    FCPWGB_CUDA(cudaMemcpyAsync(hVerts.data(), verts.ptr, hVerts.size() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                st));
    FCPWGB_CUDA(cudaStreamSynchronize(st));
    return fcpwgb_gpu_scene_transfer(s, dim == 3 ? FCPWGB_TRIANGLE_BVH : FCPWGB_LINE_SEGMENT_BVH, hNodes.data(),
                                     nNodes, hPrims.data(), nPrims, nullptr, 0, hVerts.data(), nVertices);
}

extern "C" int fcpwgb_gpu_scene_build_device(fcpwgb_gpu_scene *s, const float *positions, uint32_t n_vertices,
                                             const int32_t *indices, uint32_t n_primitives, uint32_t max_leaf_size,
                                             void *stream) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    int rc = s->activate();
    if (rc) return rc;
    return gpuBuild(s, positions, n_vertices, indices, n_primitives, max_leaf_size, s->pick(stream));
}

static int sahHeuristicOf(int aggregateType) {
    switch (aggregateType) {
        case FCPWGB_AGGREGATE_BVH_LONGEST_AXIS: return 0;
        case FCPWGB_AGGREGATE_BVH_SURFACE_AREA: return 1;
        case FCPWGB_AGGREGATE_BVH_OVERLAP_SURFACE: return 2;
        case FCPWGB_AGGREGATE_BVH_VOLUME: return 3;
        case FCPWGB_AGGREGATE_BVH_OVERLAP_VOLUME: return 4;
        default: return -1;
    }
}

extern "C" int fcpwgb_gpu_scene_build_sah_device(fcpwgb_gpu_scene *s, const float *positions, uint32_t n_vertices,
                                                 const int32_t *indices, uint32_t n_primitives, int aggregate_type,
                                                 void *stream) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    int h = sahHeuristicOf(aggregate_type);
    if (h < 0) return setError(FCPWGB_ERR_UNSUPPORTED, "the SAH build needs a BVH aggregate type (Bvh_*)");
    int rc = s->activate();
    if (rc) return rc;
    return gpuBuild(s, positions, n_vertices, indices, n_primitives, 4, s->pick(stream), h);
}

extern "C" int fcpwgb_gpu_scene_build_sah(fcpwgb_gpu_scene *s, const float *positions, uint32_t n_vertices,
                                          const int32_t *indices, uint32_t n_primitives, int aggregate_type) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    int h = sahHeuristicOf(aggregate_type);
    if (h < 0) return setError(FCPWGB_ERR_UNSUPPORTED, "the SAH build needs a BVH aggregate type (Bvh_*)");
    int rc = s->activate();
    if (rc) return rc;
    if (!positions || !indices || n_primitives == 0 || n_vertices == 0)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "non-empty positions and indices are required");
    for (uint64_t k = 0; k < (uint64_t)n_primitives * s->dim; k++)
        if (indices[k] < 0 || (uint32_t)indices[k] >= n_vertices)
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "vertex index out of range");
    DeviceBuffer pos, idx;
    if ((rc = pos.upload(positions, (size_t)n_vertices * s->dim * sizeof(float), s->stream))) return rc;
    if ((rc = idx.upload(indices, (size_t)n_primitives * s->dim * sizeof(int32_t), s->stream))) return rc;
    rc = gpuBuild(s, (const float *)pos.ptr, n_vertices, (const int32_t *)idx.ptr, n_primitives, 4, s->stream, h);
    cudaStreamSynchronize(s->stream);
    return rc;
}

extern "C" int fcpwgb_gpu_scene_build(fcpwgb_gpu_scene *s, const float *positions, uint32_t n_vertices,
                                      const int32_t *indices, uint32_t n_primitives, uint32_t max_leaf_size) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    int rc = s->activate();
    if (rc) return rc;
    if (!positions || !indices || n_primitives == 0 || n_vertices == 0)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "non-empty positions and indices are required");
    for (uint64_t k = 0; k < (uint64_t)n_primitives * s->dim; k++)
        if (indices[k] < 0 || (uint32_t)indices[k] >= n_vertices)
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "vertex index out of range");
    DeviceBuffer pos, idx;
    if ((rc = pos.upload(positions, (size_t)n_vertices * s->dim * sizeof(float), s->stream))) return rc;
    if ((rc = idx.upload(indices, (size_t)n_primitives * s->dim * sizeof(int32_t), s->stream))) return rc;
    rc = gpuBuild(s, (const float *)pos.ptr, n_vertices, (const int32_t *)idx.ptr, n_primitives, max_leaf_size,
                  s->stream);
    cudaStreamSynchronize(s->stream);
    return rc;
}

namespace fcpwgb {
int requireTree(fcpwgb_gpu_scene *s) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    if (s->inst)
        return setError(FCPWGB_ERR_UNSUPPORTED,
                        "a scene of several objects or instances takes closest point and ray queries only");
    if (!s->transferred) return setError(FCPWGB_ERR_NOT_TRANSFERRED, "transferToGPU has not been called");
    return s->activate();
}
}  // namespace fcpwgb

namespace fcpwgb {
int runRefit(fcpwgb_gpu_scene *s, cudaStream_t st) {
    FCPWGB_CUDA(cudaMemsetAsync(s->counters.ptr, 0, (size_t)s->nNodes * sizeof(uint32_t), st));
    RefitView v;
    v.dim = s->dim;
    v.snch = s->snch;
    v.nodes = (unsigned char *)s->nodes.ptr;
    v.prims = (const unsigned char *)s->prims.ptr;
    v.sils = (const unsigned char *)s->sils.ptr;
    v.parents = (const int32_t *)s->parents.ptr;
    v.leaves = (const uint32_t *)s->leaves.ptr;
    v.nLeaves = s->nLeaves;
    v.nNodes = s->nNodes;
    v.counters = (uint32_t *)s->counters.ptr;
    FCPWGB_CUDA(launchRefit(v, st));
    return s->afterRefit(st);
}
}  // namespace fcpwgb

extern "C" int fcpwgb_gpu_scene_refit(fcpwgb_gpu_scene *s, const void *primitives, const void *silhouettes) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (primitives) {
        if (s->dim == 3) {
            if ((rc = s->prims.upload(primitives, (size_t)s->nPrims * sizeof(DevTriangle), s->stream))) return rc;
        } else {
            std::vector<DevSegment2> tmp(s->nPrims);
            for (uint32_t k = 0; k < s->nPrims; k++) {
                const fcpwgb_line_segment &sg = ((const fcpwgb_line_segment *)primitives)[k];
                tmp[k].pa = make_float2(sg.pa.x, sg.pa.y);
                tmp[k].pb = make_float2(sg.pb.x, sg.pb.y);
                tmp[k].index = sg.index;
                tmp[k].pad = 0;
            }
            if ((rc = s->prims.upload(tmp.data(), tmp.size() * sizeof(DevSegment2), s->stream))) return rc;
            FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
        }
    }
    if (silhouettes && s->snch && s->nSils > 0) {
        if (s->dim == 3) {
            if ((rc = s->sils.upload(silhouettes, (size_t)s->nSils * sizeof(DevEdge), s->stream))) return rc;
        } else {
            std::vector<DevVertex2> tmp(s->nSils);
            for (uint32_t k = 0; k < s->nSils; k++) {
                const fcpwgb_vertex &v = ((const fcpwgb_vertex *)silhouettes)[k];
                tmp[k].p = make_float2(v.p.x, v.p.y);
                tmp[k].n0 = make_float2(v.n0.x, v.n0.y);
                tmp[k].n1 = make_float2(v.n1.x, v.n1.y);
                tmp[k].index = v.index;
                tmp[k].hasOneAdjacentFace = v.hasOneAdjacentFace;
            }
            if ((rc = s->sils.upload(tmp.data(), tmp.size() * sizeof(DevVertex2), s->stream))) return rc;
            FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
        }
    }
    if ((rc = runRefit(s, s->stream))) return rc;
    FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_update_vertices_device(fcpwgb_gpu_scene *s, const float *positions,
                                                       uint32_t n_vertices, void *stream) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (!s->hasTopology)
        return setError(FCPWGB_ERR_UNSUPPORTED, "the tree was transferred without prim_vertices");
    if (!positions || n_vertices != s->nVertices)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "positions must hold the transferred vertex count");
    cudaStream_t st = s->pick(stream);
    FCPWGB_CUDA(launchGatherPrimitives(s->dim, positions, (const int32_t *)s->primVerts.ptr, s->nPrims,
                                       (unsigned char *)s->prims.ptr, st));
    if (s->snch && s->nSils > 0 && s->silVerts.ptr)
        FCPWGB_CUDA(launchGatherSilhouettes(s->dim, positions, (const int32_t *)s->silVerts.ptr, s->nSils,
                                            (unsigned char *)s->sils.ptr, st));
    return runRefit(s, st);
}

// ------------------------------------------------------------------ queries
// device-array entry points
extern "C" int fcpwgb_find_closest_points_device(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                 fcpwgb_interaction *out, uint32_t n, int record_normals,
                                                 void *stream) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc) return rc;
        if (n > 0 && (!spheres || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction"))) return rc;
        return instancedClosest(s, (const DevSphere *)spheres, (DevInteraction *)out, nullptr, n, record_normals,
                                s->pick(stream));
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n > 0 && (!spheres || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction"))) return rc;
    return s->closestPoints((const DevSphere *)spheres, (DevInteraction *)out, n, record_normals, s->pick(stream));
}

extern "C" int fcpwgb_intersect_rays_device(fcpwgb_gpu_scene *s, const fcpwgb_ray *rays, fcpwgb_interaction *out,
                                            uint32_t n, int occl, void *stream) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc) return rc;
        if (n > 0 && (!rays || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        if ((rc = checkAligned(rays, 8, "ray")) || (rc = checkAligned(out, 8, "interaction"))) return rc;
        return instancedRays(s, (const DevRay *)rays, (DevInteraction *)out, nullptr, n, occl, s->pick(stream));
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n > 0 && (!rays || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    if ((rc = checkAligned(rays, 8, "ray")) || (rc = checkAligned(out, 8, "interaction"))) return rc;
    return s->rays((const DevRay *)rays, (DevInteraction *)out, n, occl, s->pick(stream));
}

extern "C" int fcpwgb_intersect_spheres_device(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                               const fcpwgb_float3 *rand_nums, fcpwgb_interaction *out, uint32_t n,
                                               void *stream) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc) return rc;
        if (n > 0 && (!spheres || !rand_nums || !out))
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction")) ||
            (rc = checkAligned(rand_nums, 4, "random number")))
            return rc;
        return instancedSample(s, (const DevSphere *)spheres, (const float3 *)rand_nums, (DevInteraction *)out,
                               nullptr, n, s->pick(stream));
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n > 0 && (!spheres || !rand_nums || !out))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction")) ||
        (rc = checkAligned(rand_nums, 4, "random number")))
        return rc;
    FCPWGB_CUDA(launchSphereSampleBinary(s->view(), (const DevSphere *)spheres, (const float3 *)rand_nums,
                                         (DevInteraction *)out, n, s->pick(stream)));
    return FCPWGB_OK;
}

namespace {
// closest silhouette points of a transferred single tree on device arrays:
// queries sorted spatially with a fast-path configuration, warp packets or the
// binary kernel; with stats (zeroed, 5 words) the packets' counting variant
int silhouettesDevice(fcpwgb_gpu_scene *s, const DevSphere *q, const uint32_t *flip, DevInteraction *out, uint32_t n,
                      float sq_min_r, float precision, cudaStream_t st, unsigned long long *stats) {
    int rc;
    if (!s->snch || s->nSils == 0) {
        // no silhouette data: the reference kernel leaves every result at its default
        FCPWGB_CUDA(launchFillDefault(out, n, st));
        return FCPWGB_OK;
    }
    const uint32_t *perm = nullptr;
    if (s->useWide() && s->wideConfig.sortQueries && n >= 4096) {
        // with a fast-path configuration the queries are sorted spatially first, so
        // a warp packet holds neighbouring queries (the packets' answers, like the
        // binary kernel's, do not depend on the order of the queries)
        if ((rc = s->sortCells.ensure(sizeof(uint32_t) * kSortScratchWords))) return rc;
        if ((rc = s->sortPerm.ensure((size_t)n * sizeof(uint32_t)))) return rc;
        if ((rc = s->sortSpheres.ensure((size_t)n * sizeof(DevSphere)))) return rc;
        FCPWGB_CUDA(launchSortQueries(s->sortLimits(), q, n, (uint32_t *)s->sortCells.ptr,
                                      (DevSphere *)s->sortSpheres.ptr, (uint32_t *)s->sortPerm.ptr, s->smCount(), st));
        q = (const DevSphere *)s->sortSpheres.ptr;
        perm = (const uint32_t *)s->sortPerm.ptr;
    }
    if (s->usePacketSilhouettes(sq_min_r)) {
        uint32_t *counter = nullptr, grid = 0;
        if (s->wideConfig.persistent) {  // packets handed to the warps of one resident wave from a counter
            if ((rc = s->workCounter.ensure(16))) return rc;
            FCPWGB_CUDA(cudaMemsetAsync(s->workCounter.ptr, 0, 4, st));
            counter = (uint32_t *)s->workCounter.ptr;
            grid = std::min<uint32_t>((n + 127) / 128, (uint32_t)s->smCount() * 8u);
        }
        FCPWGB_CUDA(launchSilhouettePacket(s->view(), q, flip, perm, out, n, sq_min_r, precision, counter, grid, st,
                                           stats));
        return FCPWGB_OK;
    }
    if (stats) return setError(FCPWGB_ERR_UNSUPPORTED, "silhouette statistics count the warp packets: set a fast-path "
                                                       "configuration and a squared minimum radius <= 0");
    FCPWGB_CUDA(launchSilhouetteBinary(s->view(), q, flip, perm, out, n, sq_min_r, precision, st));
    return FCPWGB_OK;
}
}  // namespace

extern "C" int fcpwgb_find_closest_silhouette_points_device(fcpwgb_gpu_scene *s,
                                                            const fcpwgb_bounding_sphere *spheres,
                                                            const uint32_t *flip, fcpwgb_interaction *out,
                                                            uint32_t n, float sq_min_r, float precision,
                                                            void *stream) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc) return rc;
        if (n > 0 && (!spheres || !flip || !out))
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction")) ||
            (rc = checkAligned(flip, 4, "flip")))
            return rc;
        return instancedSilhouettes(s, (const DevSphere *)spheres, flip, (DevInteraction *)out, nullptr, n, sq_min_r,
                                    precision, s->pick(stream));
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n > 0 && (!spheres || !flip || !out))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction")) ||
        (rc = checkAligned(flip, 4, "flip")))
        return rc;
    return silhouettesDevice(s, (const DevSphere *)spheres, flip, (DevInteraction *)out, n, sq_min_r, precision,
                             s->pick(stream), nullptr);
}

extern "C" int fcpwgb_silhouette_traversal_stats(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                 const uint32_t *flip, fcpwgb_interaction *out, uint32_t n,
                                                 float sq_min_r, float precision, uint64_t *stats) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (!stats) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL stats");
    if (n > 0 && (!spheres || !flip || !out))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction")) ||
        (rc = checkAligned(flip, 4, "flip")))
        return rc;
    DeviceBuffer counters;
    if ((rc = counters.ensure(8 * sizeof(unsigned long long)))) return rc;
    FCPWGB_CUDA(cudaMemsetAsync(counters.ptr, 0, 8 * sizeof(unsigned long long), s->stream));
    if ((rc = silhouettesDevice(s, (const DevSphere *)spheres, flip, (DevInteraction *)out, n, sq_min_r, precision,
                                s->stream, (unsigned long long *)counters.ptr)))
        return rc;
    unsigned long long h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    FCPWGB_CUDA(cudaMemcpyAsync(h, counters.ptr, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
    stats[0] = n;
    for (int k = 0; k < 5; k++) stats[k + 1] = h[k];
    stats[6] = stats[7] = 0;
    return FCPWGB_OK;
}

// host-array entry points: stage through device buffers, run, read back, synchronise
namespace {
struct HostQuery {
    fcpwgb_gpu_scene *s;
    int begin(const void *in0, size_t b0, const void *in1, size_t b1, size_t outBytes) {
        int rc;
        if ((rc = s->qIn0.ensure(b0 > 0 ? b0 : 16))) return rc;
        if (b1 && (rc = s->qIn1.ensure(b1))) return rc;
        if ((rc = s->qOut.ensure(outBytes > 0 ? outBytes : 16))) return rc;
        if (b0) FCPWGB_CUDA(cudaMemcpyAsync(s->qIn0.ptr, in0, b0, cudaMemcpyHostToDevice, s->stream));
        if (b1) FCPWGB_CUDA(cudaMemcpyAsync(s->qIn1.ptr, in1, b1, cudaMemcpyHostToDevice, s->stream));
        return FCPWGB_OK;
    }
    int finish(void *out, size_t outBytes) {
        uint32_t err[4] = {0, 0, 0, 0};
        if (outBytes) FCPWGB_CUDA(cudaMemcpyAsync(out, s->qOut.ptr, outBytes, cudaMemcpyDeviceToHost, s->stream));
        FCPWGB_CUDA(cudaMemcpyAsync(err, s->errorWord.ptr, sizeof(err), cudaMemcpyDeviceToHost, s->stream));
        FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
        if (err[0]) {
            cudaMemsetAsync(s->errorWord.ptr, 0, sizeof(err), s->stream);
            cudaStreamSynchronize(s->stream);
            return setError(FCPWGB_ERR_TRAVERSAL, "device traversal error word " + std::to_string(err[0]));
        }
        return FCPWGB_OK;
    }
};
}  // namespace

extern "C" int fcpwgb_find_closest_points(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                          fcpwgb_interaction *out, uint32_t n, int record_normals) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc || n == 0) return rc;
        if (!spheres || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        return instancedHost(s, spheres, (size_t)n * sizeof(DevSphere), out, nullptr, n, false, record_normals);
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n == 0) return FCPWGB_OK;
    if (!spheres || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    return s->closestPointsHost(spheres, out, n, record_normals);
}

extern "C" int fcpwgb_intersect_rays(fcpwgb_gpu_scene *s, const fcpwgb_ray *rays, fcpwgb_interaction *out,
                                     uint32_t n, int occl) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc || n == 0) return rc;
        if (!rays || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        return instancedHost(s, rays, (size_t)n * sizeof(DevRay), out, nullptr, n, true, occl);
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n == 0) return FCPWGB_OK;
    if (!rays || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    HostQuery h{s};
    size_t ob = (size_t)n * sizeof(DevInteraction);
    if ((rc = h.begin(rays, (size_t)n * sizeof(DevRay), nullptr, 0, ob))) return rc;
    if ((rc = s->rays((const DevRay *)s->qIn0.ptr, (DevInteraction *)s->qOut.ptr, n, occl, s->stream))) return rc;
    return h.finish(out, ob);
}

extern "C" int fcpwgb_intersect_spheres(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                        const fcpwgb_float3 *rand_nums, fcpwgb_interaction *out, uint32_t n) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc || n == 0) return rc;
        if (!spheres || !rand_nums || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        return instancedHostQuery(s, InstancedQuery::Sample, spheres, (size_t)n * sizeof(DevSphere), rand_nums,
                                  (size_t)n * sizeof(float3), out, nullptr, n, 0, 0.0f, 0.0f);
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n == 0) return FCPWGB_OK;
    if (!spheres || !rand_nums || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    HostQuery h{s};
    size_t ob = (size_t)n * sizeof(DevInteraction);
    if ((rc = h.begin(spheres, (size_t)n * 16, rand_nums, (size_t)n * 12, ob))) return rc;
    FCPWGB_CUDA(launchSphereSampleBinary(s->view(), (const DevSphere *)s->qIn0.ptr, (const float3 *)s->qIn1.ptr,
                                         (DevInteraction *)s->qOut.ptr, n, s->stream));
    return h.finish(out, ob);
}

extern "C" int fcpwgb_find_closest_silhouette_points(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                     const uint32_t *flip, fcpwgb_interaction *out, uint32_t n,
                                                     float sq_min_r, float precision) {
    if (s && s->inst) {
        int rc = s->activate();
        if (rc || n == 0) return rc;
        if (!spheres || !flip || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
        return instancedHostQuery(s, InstancedQuery::Silhouette, spheres, (size_t)n * sizeof(DevSphere), flip,
                                  (size_t)n * sizeof(uint32_t), out, nullptr, n, 0, sq_min_r, precision);
    }
    int rc = requireTree(s);
    if (rc) return rc;
    if (n == 0) return FCPWGB_OK;
    if (!spheres || !flip || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    HostQuery h{s};
    size_t ob = (size_t)n * sizeof(DevInteraction);
    if ((rc = h.begin(spheres, (size_t)n * 16, flip, (size_t)n * 4, ob))) return rc;
    rc = fcpwgb_find_closest_silhouette_points_device(s, (const fcpwgb_bounding_sphere *)s->qIn0.ptr,
                                                      (const uint32_t *)s->qIn1.ptr,
                                                      (fcpwgb_interaction *)s->qOut.ptr, n, sq_min_r, precision,
                                                      s->stream);
    if (rc) return rc;
    return h.finish(out, ob);
}

extern "C" int fcpwgb_closest_points_traversal_stats(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                     fcpwgb_interaction *out, uint32_t n, uint64_t *stats) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (!stats) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL stats");
    if (n > 0 && (!spheres || !out)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(out, 8, "interaction"))) return rc;
    DeviceBuffer counters;
    if ((rc = counters.ensure(8 * sizeof(unsigned long long)))) return rc;
    FCPWGB_CUDA(cudaMemsetAsync(counters.ptr, 0, 8 * sizeof(unsigned long long), s->stream));
    if ((rc = s->closestPointsStats((const DevSphere *)spheres, (DevInteraction *)out, n,
                                    (unsigned long long *)counters.ptr, s->stream)))
        return rc;
    unsigned long long h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    FCPWGB_CUDA(cudaMemcpyAsync(h, counters.ptr, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
    stats[0] = n;
    for (int k = 0; k < 5; k++) stats[k + 1] = h[k];
    stats[6] = stats[7] = 0;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_set_traversal(fcpwgb_gpu_scene *s, const fcpwgb_traversal_config *c) {
    if (!s || !c) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!(c->branching == 0 || c->branching == 2 || c->branching == 4 || c->branching == 8))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "branching must be 0, 2, 4 or 8");
    if (!(c->bits == 8 || c->bits == 16 || c->bits == 32))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "bits must be 8, 16 or 32");
    if (c->block_size != 128) return setError(FCPWGB_ERR_UNSUPPORTED, "the wide kernels run 128-thread blocks");
    if (c->leaf_size < 0 || c->leaf_size > 15) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "leaf_size must be 0..15");
    if (c->short_stack != 0 && c->short_stack != 16)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "short_stack must be 0 or 16");
    if (!(c->threads_per_query == 1 || c->threads_per_query == 2 || c->threads_per_query == 4 ||
          c->threads_per_query == 8))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "threads_per_query must be 1, 2, 4 or 8");
    if (c->threads_per_query > 1 && c->packet)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "threads_per_query > 1 and packet are exclusive");
    WideConfig w;
    w.branching = c->branching;
    w.bits = c->bits;
    w.blockSize = c->block_size;
    w.sortQueries = c->sort_queries != 0;
    w.persistent = c->persistent != 0;
    w.precise = c->precise != 0;
    w.packet = c->packet != 0;
    w.leafSize = c->leaf_size;
    w.shortStack = c->short_stack;
    w.lanes = c->threads_per_query;
    s->wideConfig = w;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_get_traversal(const fcpwgb_gpu_scene *s, fcpwgb_traversal_config *c) {
    if (!s || !c) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    c->branching = s->wideConfig.branching;
    c->bits = s->wideConfig.bits;
    c->block_size = s->wideConfig.blockSize;
    c->sort_queries = s->wideConfig.sortQueries;
    c->persistent = s->wideConfig.persistent;
    c->precise = s->wideConfig.precise;
    c->packet = s->wideConfig.packet;
    c->leaf_size = s->wideConfig.leafSize;
    c->short_stack = s->wideConfig.shortStack;
    c->threads_per_query = s->wideConfig.lanes;
    return FCPWGB_OK;
}

// ------------------------------------------------------------- gradients
static int gradView(fcpwgb_gpu_scene *s, GradView &gv) {
    if (!s->hasTopology)
        return setError(FCPWGB_ERR_UNSUPPORTED, "gradients need the tree transferred with prim_vertices");
    int rc;
    if ((rc = s->gradCorners.ensure((size_t)s->nPrims * s->dim * 3 * sizeof(long long)))) return rc;
    if ((rc = s->gradMax.ensure(16))) return rc;
    gv.dim = s->dim;
    gv.nPrims = s->nPrims;
    gv.nVertices = s->nVertices;
    gv.origVerts = (const int32_t *)s->origVerts.ptr;
    gv.csrOff = (const uint32_t *)s->csrOff.ptr;
    gv.csrCorner = (const uint32_t *)s->csrCorner.ptr;
    gv.corners = (long long *)s->gradCorners.ptr;
    gv.maxBits = (unsigned int *)s->gradMax.ptr;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_closest_point_backward_device(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                    const fcpwgb_interaction *forward, const float *grad_d,
                                                    uint32_t n, float *grad_x, float *grad_vertices, void *stream) {
    int rc = requireTree(s);
    if (rc) return rc;
    if ((n > 0 && (!spheres || !forward || !grad_d || !grad_x)) || !grad_vertices)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL array");
    if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(forward, 8, "interaction"))) return rc;
    GradView gv;
    if ((rc = gradView(s, gv))) return rc;
    FCPWGB_CUDA(launchDistanceBackward(gv, (const DevSphere *)spheres, (const DevInteraction *)forward, grad_d, n,
                                       grad_x, grad_vertices, s->pick(stream)));
    return FCPWGB_OK;
}

extern "C" int fcpwgb_ray_backward_device(fcpwgb_gpu_scene *s, const fcpwgb_ray *rays,
                                          const fcpwgb_interaction *forward, const float *grad_t, uint32_t n,
                                          float *grad_o, float *grad_dir, float *grad_vertices, void *stream) {
    int rc = requireTree(s);
    if (rc) return rc;
    if ((n > 0 && (!rays || !forward || !grad_t || !grad_o || !grad_dir)) || !grad_vertices)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL array");
    if ((rc = checkAligned(rays, 8, "ray")) || (rc = checkAligned(forward, 8, "interaction"))) return rc;
    GradView gv;
    if ((rc = gradView(s, gv))) return rc;
    FCPWGB_CUDA(launchRayBackward(gv, (const DevRay *)rays, (const DevInteraction *)forward, grad_t, n, grad_o,
                                  grad_dir, grad_vertices, s->pick(stream)));
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_enable_kernel_timing(fcpwgb_gpu_scene *s, int enable) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    s->timing = enable != 0;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_kernel_time(fcpwgb_gpu_scene *s, double *total_ms, uint32_t *launches) {
    if (!s || !total_ms || !launches) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = s->activate();
    if (rc) return rc;
    double sum = 0.0;
    for (auto &p : s->timedEvents) {
        FCPWGB_CUDA(cudaEventSynchronize(p.second));
        float ms = 0.0f;
        FCPWGB_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
        sum += ms;
    }
    *total_ms = sum;
    *launches = (uint32_t)s->timedEvents.size();
    s->freeEvents.insert(s->freeEvents.end(), s->timedEvents.begin(), s->timedEvents.end());
    s->timedEvents.clear();
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_info(fcpwgb_gpu_scene *s, fcpwgb_bvh_info *info) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (!info) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL info");
    info->dim = s->dim;
    info->bvh_type = s->dim == 3 ? (s->snch ? FCPWGB_TRIANGLE_SNCH : FCPWGB_TRIANGLE_BVH)
                                 : (s->snch ? FCPWGB_LINE_SEGMENT_SNCH : FCPWGB_LINE_SEGMENT_BVH);
    info->n_nodes = s->nNodes;
    info->n_leaves = s->nLeaves;
    info->max_depth = s->maxDepth;
    info->n_primitives = s->nPrims;
    info->n_silhouettes = s->nSils;
    info->n_vertices = s->nVertices;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_export_nodes(fcpwgb_gpu_scene *s, void *nodes) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (!nodes) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL nodes");
    size_t stride = s->snch ? 64 : 32;
    std::vector<unsigned char> h((size_t)s->nNodes * stride);
    FCPWGB_CUDA(cudaMemcpyAsync(h.data(), s->nodes.ptr, h.size(), cudaMemcpyDeviceToHost, s->stream));
    FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
    for (uint32_t i = 0; i < s->nNodes; i++) {
        const unsigned char *d = h.data() + (size_t)i * stride;
        if (s->snch) {
            fcpwgb_snch_node &o = ((fcpwgb_snch_node *)nodes)[i];
            std::memcpy(&o.box, d, 24);
            std::memcpy(&o.nPrimitives, d + 24, 4);
            std::memcpy(&o.offset, d + 28, 4);
            std::memcpy(&o.cone, d + 32, 20);
            std::memcpy(&o.nSilhouettes, d + 52, 4);
            std::memcpy(&o.silhouetteOffset, d + 56, 4);
        } else {
            std::memcpy((unsigned char *)nodes + (size_t)i * 32, d, 32);
        }
    }
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_check_errors(fcpwgb_gpu_scene *s, uint32_t *error_word) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    int rc = s->activate();
    if (rc) return rc;
    uint32_t err[4] = {0, 0, 0, 0};
    FCPWGB_CUDA(cudaMemcpyAsync(err, s->errorWord.ptr, sizeof(err), cudaMemcpyDeviceToHost, s->stream));
    FCPWGB_CUDA(cudaMemsetAsync(s->errorWord.ptr, 0, sizeof(err), s->stream));
    FCPWGB_CUDA(cudaStreamSynchronize(s->stream));
    if (error_word) *error_word = err[0];
    return FCPWGB_OK;
}

extern "C" int fcpwgb_closest_distances_f64_device(fcpwgb_gpu_scene *s, const fcpwgb_bounding_sphere *spheres,
                                                   uint32_t n, double *distances, void *stream) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (n > (1u << 24)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "at most 2^24 queries per brute-force call");
    if (n && (!spheres || !distances)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL array");
    if ((rc = checkAligned(spheres, 16, "sphere"))) return rc;
    FCPWGB_CUDA(launchBruteF64(s->dim, (const unsigned char *)s->prims.ptr, s->nPrims, (const DevSphere *)spheres, n,
                               distances, s->pick(stream)));
    return FCPWGB_OK;
}

// --------------------------------------------- contains / line of sight
extern "C" int fcpwgb_contains_device(fcpwgb_gpu_scene *s, const fcpwgb_float3 *points, uint32_t n, uint32_t *result,
                                      void *stream) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (n > 0 && (!points || !result)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL point or result array");
    return s->containsPoints((const float *)points, n, result, s->pick(stream));
}

extern "C" int fcpwgb_contains(fcpwgb_gpu_scene *s, const fcpwgb_float3 *points, uint32_t n, uint32_t *result) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (n == 0) return FCPWGB_OK;
    if (!points || !result) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL point or result array");
    HostQuery h{s};
    size_t ob = (size_t)n * sizeof(uint32_t);
    if ((rc = h.begin(points, (size_t)n * 12, nullptr, 0, ob))) return rc;
    if ((rc = s->containsPoints((const float *)s->qIn0.ptr, n, (uint32_t *)s->qOut.ptr, s->stream))) return rc;
    return h.finish(result, ob);
}

extern "C" int fcpwgb_has_line_of_sight_device(fcpwgb_gpu_scene *s, const fcpwgb_float3 *points_a,
                                               const fcpwgb_float3 *points_b, uint32_t n, uint32_t *result,
                                               void *stream) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (n > 0 && (!points_a || !points_b || !result))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL point or result array");
    FCPWGB_CUDA(launchLineOfSight(s->view(), (const float *)points_a, (const float *)points_b, n, result,
                                  s->pick(stream)));
    return FCPWGB_OK;
}

extern "C" int fcpwgb_has_line_of_sight(fcpwgb_gpu_scene *s, const fcpwgb_float3 *points_a,
                                        const fcpwgb_float3 *points_b, uint32_t n, uint32_t *result) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (n == 0) return FCPWGB_OK;
    if (!points_a || !points_b || !result) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL point or result array");
    HostQuery h{s};
    size_t ob = (size_t)n * sizeof(uint32_t);
    if ((rc = h.begin(points_a, (size_t)n * 12, points_b, (size_t)n * 12, ob))) return rc;
    FCPWGB_CUDA(launchLineOfSight(s->view(), (const float *)s->qIn0.ptr, (const float *)s->qIn1.ptr, n,
                                  (uint32_t *)s->qOut.ptr, s->stream));
    return h.finish(result, ob);
}
