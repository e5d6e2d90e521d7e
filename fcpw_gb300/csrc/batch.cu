// Batches of scenes: many meshes of uneven size, each with its own query set,
// answered by one persistent launch.
//
// The wide trees of all scenes are concatenated into one forest (inner child
// references and leaf offsets rebased, so every record addresses the forest
// directly) and the primitives into one array. The queries arrive grouped by
// scene (offsets[s] .. offsets[s+1]); one counting sort orders them by
// (scene, Hilbert index of the cell in that scene's own grid) and records each query's
// root, and the wide kernel -- persistent blocks taking neighbouring queries
// from a work counter -- starts every query at its scene's root. The
// sequence (clears, sort, traversal) is captured once in a CUDA graph and
// replayed by later calls with the same buffers, so a call costs one graph
// launch.
#include <algorithm>
#include <cstring>
#include <thread>

#include "host_bvh.h"
#include "scene.h"

using namespace fcpwgb;

namespace {

struct BatchScene {
    std::vector<uint32_t> nP, off;     // binary tree
    std::vector<float> boxes;
    std::vector<unsigned char> prims;  // 48 B triangles (3D) / 24 B segments (2D), leaf order
    uint32_t nPrims = 0;
    float box[6];
};

struct GraphKey {
    const void *spheres, *out, *nodes, *prims, *cells, *perm, *sorted, *roots, *grids, *offsets, *sel;
    uint32_t n, recordNormal, branching, bits, persistent, precise, sort, packet, leaf, shortStack, lanes;
    bool operator==(const GraphKey &o) const { return std::memcmp(this, &o, sizeof(GraphKey)) == 0; }
};

constexpr uint32_t kMaxBatchCells = 1u << 26;

}  // namespace

struct fcpwgb_gpu_batch {
    int dim = 3, device = 0, numSMs = 1;
    cudaStream_t stream = nullptr;  // private: graph capture and host-array calls
    std::vector<BatchScene> scenes;
    WideConfig cfg;
    bool useGraph = true;

    // forest of the current (branching, bits)
    bool forestValid = false;
    int forestW = 0, forestBits = 0, forestLeaf = 0;
    uint32_t nNodes = 0, nPrims = 0;
    std::vector<uint32_t> roots;
    DeviceBuffer nodes, prims;

    // query layout of the current offsets
    std::vector<uint32_t> hostOffsets;
    std::vector<BatchSceneGrid> grids;
    uint32_t nCells = 0;
    DeviceBuffer gridBuf, offsetBuf, cells, tileSums, perm, sorted, rootBuf, counter, errorWord;
    DeviceBuffer refineSel;  // precise mode on triangles: winner and runner-up leaf positions per sorted query
    DeviceBuffer qIn, qOut;

    cudaGraphExec_t exec = nullptr;
    GraphKey key;

    ~fcpwgb_gpu_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (stream) cudaStreamDestroy(stream);
    }
    void dropGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
    }
};

namespace {

int activate(const fcpwgb_gpu_batch *b) {
    cudaError_t e = cudaSetDevice(b->device);
    return e == cudaSuccess ? FCPWGB_OK : cudaFail(e, "cudaSetDevice");
}

// collapse every scene to (W, bits) on the host (scenes in parallel), rebase
// and concatenate; upload the forest
int ensureForest(fcpwgb_gpu_batch *b) {
    const int W = b->cfg.branching, bits = b->cfg.bits, leaf = b->cfg.leafSize;
    if (b->forestValid && b->forestW == W && b->forestBits == bits && b->forestLeaf == leaf) return FCPWGB_OK;
    if (b->scenes.empty()) return setError(FCPWGB_ERR_NOT_TRANSFERRED, "the batch holds no scenes");
    // invalid until the rebuild completes: a failed allocation releases the old buffers
    b->forestValid = false;
    b->hostOffsets.clear();  // the layout records roots of the forest
    const size_t nS = b->scenes.size();
    std::vector<WideHost> wide(nS);
    std::vector<char> ok(nS, 0);
    unsigned nThreads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
    nThreads = (unsigned)std::min<size_t>(nThreads, nS);
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nThreads; t++)
        pool.emplace_back([&, t]() {
            for (size_t s = t; s < nS; s += nThreads)
                ok[s] = buildWideTree(W, bits, b->scenes[s].nP, b->scenes[s].off, b->scenes[s].boxes, wide[s], leaf);
        });
    for (auto &th : pool) th.join();
    for (size_t s = 0; s < nS; s++)
        if (!ok[s])
            return setError(FCPWGB_ERR_UNSUPPORTED, "scene " + std::to_string(s) +
                                                        " cannot be collapsed into the requested wide layout");
    const size_t nb = (size_t)wideNodeBytes(W, bits);
    uint64_t totalNodes = 0, totalPrims = 0, primBytes = b->dim == 3 ? 48 : 24;
    for (size_t s = 0; s < nS; s++) {
        totalNodes += wide[s].nNodes;
        totalPrims += b->scenes[s].nPrims;
    }
    if (totalNodes >= (1ull << 31) || totalPrims >= (1ull << 27))
        return setError(FCPWGB_ERR_UNSUPPORTED, "the batch exceeds 2^31 wide records or 2^27 primitives");
    std::vector<unsigned char> hNodes(totalNodes * nb), hPrims(totalPrims * primBytes);
    b->roots.assign(nS, 0);
    uint32_t nodeBase = 0, primBase = 0;
    for (size_t s = 0; s < nS; s++) {
        const WideHost &w = wide[s];
        b->roots[s] = nodeBase;
        for (uint32_t i = 0; i < w.nNodes; i++) {
            unsigned char *rec = hNodes.data() + ((size_t)nodeBase + i) * nb;
            std::memcpy(rec, w.nodes.data() + (size_t)i * nb, nb);
            uint32_t ref[8];
            uint8_t cnt[8];
            std::memcpy(ref, rec + wideHeaderBytes(bits), 4 * W);
            std::memcpy(cnt, rec + wideCntOffset(W, bits), W);
            for (int c = 0; c < W; c++) {
                if (cnt[c] == kWideEmpty) continue;
                ref[c] += cnt[c] == 0 ? nodeBase : primBase;
            }
            std::memcpy(rec + wideHeaderBytes(bits), ref, 4 * W);
        }
        std::memcpy(hPrims.data() + (size_t)primBase * primBytes, b->scenes[s].prims.data(),
                    b->scenes[s].prims.size());
        nodeBase += w.nNodes;
        primBase += b->scenes[s].nPrims;
    }
    int rc;
    b->dropGraph();
    if ((rc = b->nodes.upload(hNodes.data(), hNodes.size(), b->stream))) return rc;
    if ((rc = b->prims.upload(hPrims.data(), hPrims.size(), b->stream))) return rc;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cudaFail(e, "forest upload");
    b->forestValid = true;
    b->forestW = W;
    b->forestBits = bits;
    b->forestLeaf = leaf;
    b->nNodes = (uint32_t)totalNodes;
    b->nPrims = (uint32_t)totalPrims;
    for (size_t s = 0; s < b->grids.size() && s < nS; s++) b->grids[s].root = b->roots[s];
    if (!b->grids.empty()) {
        if ((rc = b->gridBuf.upload(b->grids.data(), b->grids.size() * sizeof(BatchSceneGrid), b->stream))) return rc;
        if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cudaFail(e, "grid upload");
    }
    return FCPWGB_OK;
}

// per-scene sort grids sized by the scene's query count (about 2 queries a
// cell of the grid, which spans the scene box grown by half its largest
// extent on every side; queries farther out fall into its border cells), at
// most 2^8 cells per axis in 3D and 2^12 in 2D; fine cells keep the queries
// of a warp packet close together. The density halves until the cells of all
// scenes fit kMaxBatchCells. On the 512-mesh batch (60M queries) the
// packets went from 99 to 66 ms against 16 queries a cell of a grid 3 times
// the extent.
int ensureLayout(fcpwgb_gpu_batch *b, const uint32_t *offsets, uint32_t nOffsets) {
    const uint32_t nS = (uint32_t)b->scenes.size();
    if (!offsets || nOffsets != nS + 1)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "query_offsets must hold one entry per scene plus one");
    if (b->hostOffsets.size() == nOffsets &&
        std::memcmp(b->hostOffsets.data(), offsets, nOffsets * sizeof(uint32_t)) == 0)
        return FCPWGB_OK;
    if (offsets[0] != 0) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "query_offsets[0] must be 0");
    b->hostOffsets.clear();  // no layout until this one is complete (a failed allocation releases buffers)
    for (uint32_t s = 0; s < nS; s++)
        if (offsets[s + 1] < offsets[s])
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "query_offsets must be non-decreasing");
    const uint32_t n = offsets[nS];
    std::vector<BatchSceneGrid> grids(nS);
    const int maxBits = b->dim == 3 ? 8 : 12;
    std::vector<int> bits(nS);
    uint64_t cellBase = 0;
    for (uint64_t per = 2;; per *= 2) {
        cellBase = 0;
        for (uint32_t s = 0; s < nS; s++) {
            const uint64_t nq = offsets[s + 1] - offsets[s];
            int k = 0;
            while (k < maxBits && (per << (b->dim * (k + 1))) <= nq) k++;
            bits[s] = k;
            cellBase += (uint64_t)1 << (b->dim * k);
        }
        if (cellBase <= kMaxBatchCells || per > (1ull << 32)) break;  // one cell a scene: checked below
    }
    cellBase = 0;
    for (uint32_t s = 0; s < nS; s++) {
        const int bitsPerAxis = bits[s];
        const float *bx = b->scenes[s].box;
        float ext = 1e-6f;
        for (int a = 0; a < b->dim; a++) ext = std::max(ext, bx[3 + a] - bx[a]);
        float side = 2.0f * ext, inv = (float)(1u << bitsPerAxis) / side;
        BatchSceneGrid &g = grids[s];
        g.lo = make_float3(bx[0] - 0.5f * ext, bx[1] - 0.5f * ext, b->dim == 3 ? bx[2] - 0.5f * ext : 0.0f);
        g.inv = make_float3(inv, inv, inv);
        g.cellBase = (uint32_t)cellBase;
        g.bits = (uint32_t)bitsPerAxis;
        g.root = b->forestValid ? b->roots[s] : 0u;
        g.pad = 0;
        cellBase += (uint64_t)1 << (b->dim * bitsPerAxis);
    }
    if (cellBase > kMaxBatchCells) return setError(FCPWGB_ERR_UNSUPPORTED, "too many sort cells in the batch");
    int rc;
    b->dropGraph();
    if ((rc = b->gridBuf.upload(grids.data(), grids.size() * sizeof(BatchSceneGrid), b->stream))) return rc;
    if ((rc = b->offsetBuf.upload(offsets, nOffsets * sizeof(uint32_t), b->stream))) return rc;
    if ((rc = b->cells.ensure(cellBase * sizeof(uint32_t)))) return rc;
    if ((rc = b->tileSums.ensure((size_t)batchScanTiles((uint32_t)cellBase) * sizeof(uint32_t) + 16))) return rc;
    if ((rc = b->perm.ensure((size_t)std::max(n, 1u) * sizeof(uint32_t)))) return rc;
    if ((rc = b->sorted.ensure((size_t)std::max(n, 1u) * sizeof(DevSphere)))) return rc;
    if (b->dim == 3 && (rc = b->refineSel.ensure((size_t)std::max(n, 1u) * sizeof(uint2)))) return rc;
    if ((rc = b->rootBuf.ensure((size_t)std::max(n, 1u) * sizeof(uint32_t)))) return rc;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cudaFail(e, "layout upload");
    b->grids = grids;
    b->hostOffsets.assign(offsets, offsets + nOffsets);
    b->nCells = (uint32_t)cellBase;
    return FCPWGB_OK;
}

// enqueues clears, sort and traversal on st
int enqueue(fcpwgb_gpu_batch *b, const DevSphere *spheres, DevInteraction *out, uint32_t n, int recordNormal,
            unsigned long long *stats, cudaStream_t st) {
    const uint32_t nS = (uint32_t)b->scenes.size();
    WideLaunch l;
    l.nodes = (const unsigned char *)b->nodes.ptr;
    l.prims = (const unsigned char *)b->prims.ptr;
    l.out = out;
    l.n = n;
    l.recordNormal = recordNormal;
    l.errorWord = (uint32_t *)b->errorWord.ptr;
    l.stats = stats;
    cudaError_t e = launchSortBatchQueries(b->dim, (const BatchSceneGrid *)b->gridBuf.ptr,
                                           (const uint32_t *)b->offsetBuf.ptr, nS, spheres, n,
                                           (uint32_t *)b->cells.ptr, b->nCells, (uint32_t *)b->tileSums.ptr,
                                           (DevSphere *)b->sorted.ptr, (uint32_t *)b->perm.ptr,
                                           (uint32_t *)b->rootBuf.ptr, st);
    if (e != cudaSuccess) return cudaFail(e, "batch sort");
    l.spheres = (const DevSphere *)b->sorted.ptr;
    l.perm = (const uint32_t *)b->perm.ptr;
    l.roots = (const uint32_t *)b->rootBuf.ptr;
    l.sel = (uint2 *)b->refineSel.ptr;
    uint32_t blocks = (n + 127) / 128;
    l.packet = b->cfg.packet;
    l.shortStack = b->cfg.shortStack;
    l.lanes = b->cfg.lanes;
    if (b->cfg.persistent && b->cfg.lanes == 1) {
        if ((e = cudaMemsetAsync(b->counter.ptr, 0, 4, st)) != cudaSuccess) return cudaFail(e, "memset");
        l.counter = (uint32_t *)b->counter.ptr;
        blocks = std::min<uint32_t>(blocks, (uint32_t)b->numSMs * 8u);
    }
    l.grid = blocks;
    if ((e = launchWide(b->cfg.branching, b->cfg.bits, b->dim, b->cfg.precise != 0, l, st)) != cudaSuccess)
        return cudaFail(e, "batch closest point launch");
    return FCPWGB_OK;
}

int prepare(fcpwgb_gpu_batch *b, const uint32_t *offsets, uint32_t nOffsets) {
    int rc = activate(b);
    if (rc) return rc;
    if ((rc = ensureForest(b))) return rc;
    return ensureLayout(b, offsets, nOffsets);
}

int runDevice(fcpwgb_gpu_batch *b, const DevSphere *spheres, const uint32_t *offsets, uint32_t nOffsets,
              DevInteraction *out, int recordNormal, cudaStream_t st) {
    int rc = prepare(b, offsets, nOffsets);
    if (rc) return rc;
    const uint32_t n = b->hostOffsets.back();
    if (n == 0) return FCPWGB_OK;
    if (!spheres || !out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    if (!b->useGraph) return enqueue(b, spheres, out, n, recordNormal, nullptr, st);
    GraphKey k;
    std::memset(&k, 0, sizeof(k));
    k.spheres = spheres; k.out = out; k.nodes = b->nodes.ptr; k.prims = b->prims.ptr; k.cells = b->cells.ptr;
    k.perm = b->perm.ptr; k.sorted = b->sorted.ptr; k.roots = b->rootBuf.ptr; k.grids = b->gridBuf.ptr;
    k.offsets = b->offsetBuf.ptr; k.sel = b->refineSel.ptr; k.n = n; k.recordNormal = (uint32_t)recordNormal;
    k.branching = (uint32_t)b->cfg.branching; k.bits = (uint32_t)b->cfg.bits;
    k.persistent = (uint32_t)b->cfg.persistent; k.precise = (uint32_t)b->cfg.precise;
    k.sort = (uint32_t)b->cfg.sortQueries;
    k.packet = (uint32_t)b->cfg.packet;
    k.leaf = (uint32_t)b->cfg.leafSize;
    k.shortStack = (uint32_t)b->cfg.shortStack;
    k.lanes = (uint32_t)b->cfg.lanes;
    cudaError_t e;
    if (!b->exec || !(k == b->key)) {
        b->dropGraph();
        if ((e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cudaFail(e, "cudaStreamBeginCapture");
        rc = enqueue(b, spheres, out, n, recordNormal, nullptr, b->stream);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cudaFail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return cudaFail(e, "cudaGraphInstantiate");
        }
        b->key = k;
    }
    if ((e = cudaGraphLaunch(b->exec, st)) != cudaSuccess) return cudaFail(e, "cudaGraphLaunch");
    return FCPWGB_OK;
}

}  // namespace

extern "C" int fcpwgb_gpu_batch_create(int dim, int device, fcpwgb_gpu_batch **out) {
    if (!out) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (dim != 2 && dim != 3) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return setError(FCPWGB_ERR_CUDA, "no CUDA device");
    }
    if (device < 0 || device >= count) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    auto *b = new fcpwgb_gpu_batch;
    b->dim = dim;
    b->device = device;
    b->cfg.branching = 8;
    b->cfg.bits = 8;
    int rc = activate(b);
    cudaError_t e = cudaSuccess;
    if (!rc && (e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
        rc = cudaFail(e, "cudaStreamCreate");
    if (!rc) rc = b->errorWord.ensure(16);
    if (!rc) rc = b->counter.ensure(16);
    if (!rc && (e = cudaMemset(b->errorWord.ptr, 0, 16)) != cudaSuccess) rc = cudaFail(e, "cudaMemset");
    if (!rc) {
        cudaDeviceGetAttribute(&b->numSMs, cudaDevAttrMultiProcessorCount, device);
        if (b->numSMs <= 0) b->numSMs = 1;
    }
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return FCPWGB_OK;
}

extern "C" void fcpwgb_gpu_batch_destroy(fcpwgb_gpu_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    delete b;
}

extern "C" int fcpwgb_gpu_batch_set_scenes(fcpwgb_gpu_batch *b, const fcpwgb_cpu_bvh *const *bvhs,
                                           uint32_t n_scenes) {
    if (!b || (!bvhs && n_scenes)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<BatchScene> scenes(n_scenes);
    for (uint32_t s = 0; s < n_scenes; s++) {
        if (!bvhs[s]) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL bvh in the scene list");
        const HostBvh &h = *bvhs[s]->bvh;
        if (h.dim() != b->dim) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "scene dimension does not match the batch");
        BatchScene &sc = scenes[s];
        binaryTreeArrays(h, sc.nP, sc.off, sc.boxes);
        std::memcpy(sc.box, sc.boxes.data(), 24);
        sc.nPrims = h.nPrimitives();
        if (b->dim == 3) {
            std::vector<fcpwgb_triangle> t(sc.nPrims);
            h.exportPrimitives(t.data());
            sc.prims.resize((size_t)sc.nPrims * 48);
            for (uint32_t k = 0; k < sc.nPrims; k++) {
                float r[12] = {t[k].pa.x, t[k].pa.y, t[k].pa.z, 0.0f, t[k].pb.x, t[k].pb.y,
                               t[k].pb.z, 0.0f, t[k].pc.x, t[k].pc.y, t[k].pc.z, 0.0f};
                std::memcpy(&r[3], &t[k].index, 4);
                std::memcpy(sc.prims.data() + (size_t)k * 48, r, 48);
            }
        } else {
            std::vector<fcpwgb_line_segment> g(sc.nPrims);
            h.exportPrimitives(g.data());
            sc.prims.resize((size_t)sc.nPrims * sizeof(DevSegment2));
            for (uint32_t k = 0; k < sc.nPrims; k++) {
                DevSegment2 d;
                d.pa = make_float2(g[k].pa.x, g[k].pa.y);
                d.pb = make_float2(g[k].pb.x, g[k].pb.y);
                d.index = g[k].index;
                d.pad = 0;
                std::memcpy(sc.prims.data() + (size_t)k * sizeof(DevSegment2), &d, sizeof(d));
            }
        }
    }
    int rc = activate(b);
    if (rc) return rc;
    b->dropGraph();
    b->scenes.swap(scenes);
    b->forestValid = false;
    b->hostOffsets.clear();
    b->grids.clear();
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_batch_set_traversal(fcpwgb_gpu_batch *b, const fcpwgb_traversal_config *c) {
    if (!b || !c) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!(c->branching == 2 || c->branching == 4 || c->branching == 8))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "a batch traverses wide trees: branching must be 2, 4 or 8");
    if (!(c->bits == 8 || c->bits == 16 || c->bits == 32))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "bits must be 8, 16 or 32");
    if (c->block_size != 0 && c->block_size != 128)
        return setError(FCPWGB_ERR_UNSUPPORTED, "block_size must be 128 (or 0 for the default)");
    if (c->leaf_size < 0 || c->leaf_size > 15) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "leaf_size must be 0..15");
    if (c->short_stack != 0 && c->short_stack != 16)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "short_stack must be 0 or 16");
    if (!(c->threads_per_query == 1 || c->threads_per_query == 2 || c->threads_per_query == 4 ||
          c->threads_per_query == 8))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "threads_per_query must be 1, 2, 4 or 8");
    if (c->threads_per_query > 1 && c->packet)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "threads_per_query > 1 and packet are exclusive");
    b->dropGraph();
    b->cfg.branching = c->branching;
    b->cfg.bits = c->bits;
    b->cfg.sortQueries = 1;  // the per-query roots come from the sort
    b->cfg.persistent = c->persistent != 0;
    b->cfg.precise = c->precise != 0;
    b->cfg.packet = c->packet != 0;
    b->cfg.leafSize = c->leaf_size;
    b->cfg.shortStack = c->short_stack;
    b->cfg.lanes = c->threads_per_query;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_batch_get_traversal(const fcpwgb_gpu_batch *b, fcpwgb_traversal_config *c) {
    if (!b || !c) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    c->branching = b->cfg.branching;
    c->bits = b->cfg.bits;
    c->block_size = 128;
    c->sort_queries = 1;
    c->persistent = b->cfg.persistent;
    c->precise = b->cfg.precise;
    c->packet = b->cfg.packet;
    c->leaf_size = b->cfg.leafSize;
    c->short_stack = b->cfg.shortStack;
    c->threads_per_query = b->cfg.lanes;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_batch_use_graph(fcpwgb_gpu_batch *b, int on) {
    if (!b) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL batch");
    b->useGraph = on != 0;
    if (!b->useGraph) b->dropGraph();
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_batch_find_closest_points_device(fcpwgb_gpu_batch *b, const fcpwgb_bounding_sphere *spheres,
                                                           const uint32_t *query_offsets, uint32_t n_offsets,
                                                           fcpwgb_interaction *interactions, int record_normals,
                                                           void *stream) {
    if (!b) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL batch");
    int rc;
    if ((rc = checkAligned(spheres, 16, "sphere")) || (rc = checkAligned(interactions, 8, "interaction"))) return rc;
    return runDevice(b, (const DevSphere *)spheres, query_offsets, n_offsets, (DevInteraction *)interactions,
                     record_normals, (cudaStream_t)stream);
}

extern "C" int fcpwgb_gpu_batch_find_closest_points(fcpwgb_gpu_batch *b, const fcpwgb_bounding_sphere *spheres,
                                                    const uint32_t *query_offsets, uint32_t n_offsets,
                                                    fcpwgb_interaction *interactions, int record_normals) {
    if (!b) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL batch");
    int rc = prepare(b, query_offsets, n_offsets);
    if (rc) return rc;
    const uint32_t n = b->hostOffsets.back();
    if (n == 0) return FCPWGB_OK;
    if (!spheres || !interactions) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL query or output array");
    size_t ib = (size_t)n * sizeof(DevSphere), ob = (size_t)n * sizeof(DevInteraction);
    if ((rc = b->qIn.ensure(ib)) || (rc = b->qOut.ensure(ob))) return rc;
    cudaError_t e = cudaMemcpyAsync(b->qIn.ptr, spheres, ib, cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpyAsync");
    if ((rc = runDevice(b, (const DevSphere *)b->qIn.ptr, query_offsets, n_offsets, (DevInteraction *)b->qOut.ptr,
                        record_normals, b->stream)))
        return rc;
    if ((e = cudaMemcpyAsync(interactions, b->qOut.ptr, ob, cudaMemcpyDeviceToHost, b->stream)) != cudaSuccess)
        return cudaFail(e, "cudaMemcpyAsync");
    uint32_t err = 0;
    if ((e = cudaMemcpyAsync(&err, b->errorWord.ptr, 4, cudaMemcpyDeviceToHost, b->stream)) != cudaSuccess)
        return cudaFail(e, "cudaMemcpyAsync");
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cudaFail(e, "cudaStreamSynchronize");
    if (err) {
        cudaMemsetAsync(b->errorWord.ptr, 0, 4, b->stream);
        cudaStreamSynchronize(b->stream);
        return setError(FCPWGB_ERR_TRAVERSAL, "device traversal error word " + std::to_string(err));
    }
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_batch_traversal_stats(fcpwgb_gpu_batch *b, const fcpwgb_bounding_sphere *spheres,
                                                const uint32_t *query_offsets, uint32_t n_offsets,
                                                fcpwgb_interaction *interactions, uint64_t stats[8]) {
    if (!b || !stats) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = prepare(b, query_offsets, n_offsets);
    if (rc) return rc;
    const uint32_t n = b->hostOffsets.back();
    DeviceBuffer counters;
    if ((rc = counters.ensure(8 * sizeof(unsigned long long)))) return rc;
    cudaError_t e = cudaMemsetAsync(counters.ptr, 0, 8 * sizeof(unsigned long long), b->stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemsetAsync");
    if (n > 0 && (rc = enqueue(b, (const DevSphere *)spheres, (DevInteraction *)interactions, n, 0,
                               (unsigned long long *)counters.ptr, b->stream)))
        return rc;
    unsigned long long h[8];
    if ((e = cudaMemcpyAsync(h, counters.ptr, sizeof(h), cudaMemcpyDeviceToHost, b->stream)) != cudaSuccess)
        return cudaFail(e, "cudaMemcpyAsync");
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cudaFail(e, "cudaStreamSynchronize");
    stats[0] = n;
    for (int k = 0; k < 5; k++) stats[k + 1] = h[k];
    stats[6] = stats[7] = 0;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_batch_info(const fcpwgb_gpu_batch *b, uint32_t *n_scenes, uint32_t *n_wide_nodes,
                                     uint32_t *n_primitives, uint32_t *n_sort_cells) {
    if (!b) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL batch");
    if (n_scenes) *n_scenes = (uint32_t)b->scenes.size();
    if (n_wide_nodes) *n_wide_nodes = b->forestValid ? b->nNodes : 0;
    if (n_primitives) {
        uint64_t t = 0;
        for (const auto &s : b->scenes) t += s.nPrims;
        *n_primitives = (uint32_t)t;
    }
    if (n_sort_cells) *n_sort_cells = b->nCells;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_batch_check_errors(fcpwgb_gpu_batch *b, uint32_t *error_word) {
    if (!b || !error_word) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = activate(b);
    if (rc) return rc;
    uint32_t w = 0;
    cudaError_t e = cudaMemcpy(&w, b->errorWord.ptr, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemcpy");
    if (w && (e = cudaMemset(b->errorWord.ptr, 0, 4)) != cudaSuccess) return cudaFail(e, "cudaMemset");
    *error_word = w;
    return FCPWGB_OK;
}
