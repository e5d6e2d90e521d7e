// Scene files: the flattened tree, primitives, silhouettes and topology of a
// host-built BVH in the interop layouts, plus any number of derived wide
// trees, so that a later process loads a scene onto the GPU without the CPU
// build and without the wide collapse.
//
// Layout (little-endian; every section starts on a 16-byte boundary):
//   header   64 B: magic "FCPWGB" 0 1, then uint32 dim, bvh_type, n_nodes,
//            n_primitives, n_silhouettes, n_vertices, has_topology, n_wide;
//            zero padding
//   nodes    n_nodes x 32 B (GPUBvhNode) or 60 B (GPUSnchNode)
//   prims    n_primitives x 40 B (GPUTriangle) or 28 B (GPULineSegment)
//   sils     n_silhouettes x 56 B (GPUEdge) or 44 B (GPUVertex)
//   topology (has_topology) n_primitives x dim int32 primitive vertices, then
//            n_silhouettes x (dim + 1) int32 silhouette vertices
//   wide     n_wide times: 16 B {uint32 branching, bits, leaf_size, n_records},
//            the records (n_records x wideNodeBytes), then n_records x
//            branching int32 binary nodes behind the slots
//   trailer  uint64 FNV-1a hash of every byte before it
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "host_bvh.h"
#include "scene.h"

using namespace fcpwgb;

extern "C" int fcpwgb_gpu_scene_transfer(fcpwgb_gpu_scene *scene, int bvh_type, const void *nodes, uint32_t n_nodes,
                                         const void *primitives, uint32_t n_primitives, const void *silhouettes,
                                         uint32_t n_silhouettes, const int32_t *prim_vertices, uint32_t n_vertices);

namespace {

const unsigned char kMagic[8] = {'F', 'C', 'P', 'W', 'G', 'B', 0, 1};

struct Header {
    unsigned char magic[8];
    uint32_t dim, bvhType, nNodes, nPrims, nSils, nVertices, hasTopology, nWide;
    uint32_t pad[6];
};
static_assert(sizeof(Header) == 64, "scene file header");

uint64_t fnv1a(const unsigned char *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

size_t nodeBytes(int bvhType) { return bvhType >= FCPWGB_LINE_SEGMENT_SNCH ? 60 : 32; }
size_t primBytes(int dim) { return dim == 3 ? 40 : 28; }
size_t silBytes(int dim) { return dim == 3 ? 56 : 44; }

struct Writer {
    std::vector<unsigned char> buf;
    void put(const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        buf.insert(buf.end(), c, c + n);
    }
    void align() { buf.resize((buf.size() + 15) / 16 * 16, 0); }
};

struct Reader {
    const std::vector<unsigned char> &buf;
    size_t pos = 0;
    bool take(void *dst, size_t n) {
        if (pos + n > buf.size() - 8) return false;
        std::memcpy(dst, buf.data() + pos, n);
        pos += n;
        return true;
    }
    const unsigned char *view(size_t n) {
        if (pos + n > buf.size() - 8) return nullptr;
        const unsigned char *p = buf.data() + pos;
        pos += n;
        return p;
    }
    void align() { pos = (pos + 15) / 16 * 16; }
};

int readFile(const char *path, std::vector<unsigned char> &buf) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return setError(FCPWGB_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < (long)(sizeof(Header) + 8)) {
        std::fclose(f);
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "not a scene file (too short)");
    }
    buf.resize((size_t)n);
    size_t got = std::fread(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    if (got != buf.size()) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "short read of the scene file");
    uint64_t stored;
    std::memcpy(&stored, buf.data() + buf.size() - 8, 8);
    if (std::memcmp(buf.data(), kMagic, 8) != 0) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "not a scene file");
    if (fnv1a(buf.data(), buf.size() - 8) != stored)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "scene file checksum mismatch (corrupt or truncated)");
    return FCPWGB_OK;
}

// parsed view of a scene file
struct Parsed {
    Header h;
    const unsigned char *nodes = nullptr, *prims = nullptr, *sils = nullptr;
    const int32_t *primVerts = nullptr, *silVerts = nullptr;
    std::vector<std::pair<int, WideHost>> wide;
};

int parse(const std::vector<unsigned char> &buf, Parsed &p, bool withWide) {
    Reader r{buf};
    if (!r.take(&p.h, sizeof(Header))) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated header");
    const Header &h = p.h;
    if (!(h.dim == 2 || h.dim == 3) || h.bvhType < 1 || h.bvhType > 4 || (h.dim == 3) != (h.bvhType % 2 == 0))
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "scene file header is inconsistent");
    const size_t nb = nodeBytes((int)h.bvhType), pb = primBytes((int)h.dim), sb = silBytes((int)h.dim);
    r.align();
    if (!(p.nodes = r.view((size_t)h.nNodes * nb))) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated nodes");
    r.align();
    if (!(p.prims = r.view((size_t)h.nPrims * pb))) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated prims");
    r.align();
    if (!(p.sils = r.view((size_t)h.nSils * sb))) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated sils");
    if (h.hasTopology) {
        r.align();
        if (!(p.primVerts = (const int32_t *)r.view((size_t)h.nPrims * h.dim * 4)))
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated topology");
        r.align();
        if (!(p.silVerts = (const int32_t *)r.view((size_t)h.nSils * (h.dim + 1) * 4)))
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated topology");
    }
    for (uint32_t k = 0; k < h.nWide; k++) {
        r.align();
        uint32_t hw[4];
        if (!r.take(hw, 16)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated wide tree");
        int W = (int)hw[0], bits = (int)hw[1], leaf = (int)hw[2];
        if (!(W == 2 || W == 4 || W == 8) || !(bits == 8 || bits == 16 || bits == 32) || leaf < 0 || leaf > 15)
            return setError(FCPWGB_ERR_INVALID_ARGUMENT, "scene file holds an unknown wide layout");
        size_t rb = (size_t)wideNodeBytes(W, bits) * hw[3];
        const unsigned char *recs = r.view(rb);
        const int32_t *cb = (const int32_t *)r.view((size_t)hw[3] * W * 4);
        if (!recs || !cb) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "truncated wide tree");
        if (withWide) {
            WideHost w;
            w.W = W;
            w.bits = bits;
            w.nNodes = hw[3];
            w.nodes.assign(recs, recs + rb);
            w.childBinary.assign(cb, cb + (size_t)hw[3] * W);
            for (int32_t b : w.childBinary)
                if (b < -1 || b >= (int32_t)h.nNodes)
                    return setError(FCPWGB_ERR_INVALID_ARGUMENT, "wide tree references a missing binary node");
            p.wide.emplace_back(leaf, std::move(w));
        }
    }
    return FCPWGB_OK;
}

}  // namespace

extern "C" int fcpwgb_cpu_bvh_save(const fcpwgb_cpu_bvh *b, const char *path, const fcpwgb_traversal_config *wide,
                                   uint32_t n_wide) {
    if (!b || !path || (n_wide && !wide)) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    const HostBvh &t = *b->bvh;
    const int dim = t.dim();
    const bool snch = t.hasSilhouettes();
    Header h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.dim = (uint32_t)dim;
    h.bvhType = (uint32_t)t.bvhType();
    h.nNodes = t.nNodes();
    h.nPrims = t.nPrimitives();
    h.nSils = snch ? t.nSilhouetteRefs() : 0;
    h.nVertices = t.nVertices();
    h.hasTopology = 1;
    h.nWide = n_wide;
    std::vector<unsigned char> nodes((size_t)h.nNodes * nodeBytes((int)h.bvhType));
    std::vector<unsigned char> prims((size_t)h.nPrims * primBytes(dim)), sils((size_t)h.nSils * silBytes(dim));
    std::vector<int32_t> primVerts((size_t)h.nPrims * dim), silVerts((size_t)h.nSils * (dim + 1));
    t.exportNodes(nodes.data());
    t.exportPrimitives(prims.data());
    if (snch) t.exportSilhouettes(sils.data());
    t.exportTopology(nullptr, primVerts.data(), nullptr, snch ? silVerts.data() : nullptr);
    Writer w;
    w.put(&h, sizeof(h));
    w.align();
    w.put(nodes.data(), nodes.size());
    w.align();
    w.put(prims.data(), prims.size());
    w.align();
    w.put(sils.data(), sils.size());
    w.align();
    w.put(primVerts.data(), primVerts.size() * 4);
    w.align();
    w.put(silVerts.data(), silVerts.size() * 4);
    if (n_wide) {
        std::vector<uint32_t> nP, off;
        std::vector<float> boxes;
        binaryTreeArrays(t, nP, off, boxes);
        for (uint32_t k = 0; k < n_wide; k++) {
            const fcpwgb_traversal_config &c = wide[k];
            WideHost wt;
            if (!buildWideTree(c.branching, c.bits, nP, off, boxes, wt, c.leaf_size))
                return setError(FCPWGB_ERR_UNSUPPORTED, "this tree cannot be collapsed into a requested wide layout");
            uint32_t hw[4] = {(uint32_t)c.branching, (uint32_t)c.bits, (uint32_t)c.leaf_size, wt.nNodes};
            w.align();
            w.put(hw, 16);
            w.put(wt.nodes.data(), wt.nodes.size());
            w.put(wt.childBinary.data(), wt.childBinary.size() * 4);
        }
    }
    w.align();
    uint64_t hash = fnv1a(w.buf.data(), w.buf.size());
    w.put(&hash, 8);
    FILE *f = std::fopen(path, "wb");
    if (!f) return setError(FCPWGB_ERR_INVALID_ARGUMENT, std::string("cannot create ") + path);
    size_t put = std::fwrite(w.buf.data(), 1, w.buf.size(), f);
    int closed = std::fclose(f);
    if (put != w.buf.size() || closed != 0) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "short write of the scene file");
    return FCPWGB_OK;
}

extern "C" int fcpwgb_scene_file_info(const char *path, fcpwgb_bvh_info *info, uint32_t *n_wide) {
    if (!path) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL path");
    std::vector<unsigned char> buf;
    int rc = readFile(path, buf);
    if (rc) return rc;
    Parsed p;
    if ((rc = parse(buf, p, false))) return rc;
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->dim = (int)p.h.dim;
        info->bvh_type = (int)p.h.bvhType;
        info->n_nodes = p.h.nNodes;
        info->n_primitives = p.h.nPrims;
        info->n_silhouettes = p.h.nSils;
        info->n_vertices = p.h.nVertices;
    }
    if (n_wide) *n_wide = p.h.nWide;
    return FCPWGB_OK;
}

extern "C" int fcpwgb_gpu_scene_load(fcpwgb_gpu_scene *s, const char *path) {
    if (!s || !path) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<unsigned char> buf;
    int rc = readFile(path, buf);
    if (rc) return rc;
    Parsed p;
    if ((rc = parse(buf, p, true))) return rc;
    if ((int)p.h.dim != s->dim) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "scene file dimension does not match");
    // the binary tree goes through the validating transfer
    if ((rc = fcpwgb_gpu_scene_transfer(s, (int)p.h.bvhType, p.nodes, p.h.nNodes, p.prims, p.h.nPrims,
                                        p.h.nSils ? p.sils : nullptr, p.h.nSils, p.primVerts, p.h.nVertices)))
        return rc;
    if (p.silVerts && p.h.nSils) {
        if ((rc = s->silVerts.upload(p.silVerts, (size_t)p.h.nSils * (p.h.dim + 1) * 4, s->stream))) return rc;
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return cudaFail(e, "silhouette topology upload");
    }
    // a wide tree must be a tree over this binary tree: every record but the
    // root referenced exactly once and only by a record before it (so the
    // traversal cannot cycle), its slots' binary nodes exist (checked in
    // parse) and its leaves cover every primitive once
    for (auto &wt : p.wide) {
        std::vector<int> covered(p.h.nPrims, 0), referenced;
        const WideHost &w = wt.second;
        const size_t rb = (size_t)wideNodeBytes(w.W, w.bits);
        if (w.nNodes == 0) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "empty wide tree");
        referenced.assign(w.nNodes, 0);
        for (uint32_t i = 0; i < w.nNodes; i++) {
            const unsigned char *rec = w.nodes.data() + i * rb;
            uint32_t ref[8];
            uint8_t cnt[8];
            std::memcpy(ref, rec + wideHeaderBytes(w.bits), 4 * w.W);
            std::memcpy(cnt, rec + wideCntOffset(w.W, w.bits), w.W);
            for (int c = 0; c < w.W; c++) {
                if (cnt[c] == kWideEmpty) continue;
                if (cnt[c] == 0) {
                    if (ref[c] <= i || ref[c] >= w.nNodes || referenced[ref[c]]++)
                        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "wide tree is inconsistent");
                    continue;
                }
                if ((uint64_t)ref[c] + cnt[c] > p.h.nPrims)
                    return setError(FCPWGB_ERR_INVALID_ARGUMENT, "wide tree is inconsistent");
                for (uint32_t k = 0; k < cnt[c]; k++) covered[ref[c] + k]++;
            }
        }
        for (int c : covered)
            if (c != 1) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "wide tree does not cover the primitives once");
        for (uint32_t i = 1; i < w.nNodes; i++)
            if (referenced[i] != 1) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "wide tree is inconsistent");
    }
    s->preloadedWide = std::move(p.wide);
    return FCPWGB_OK;
}
