// Launch interface between the C ABI (capi.cu) and the kernel translation units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace fcpwgb {

// Device view of one transferred binary tree.
struct SceneView {
    int dim = 3;
    bool snch = false;
    const unsigned char *nodes = nullptr;  // 32 B (BVH) or 64 B (SNCH) records
    const unsigned char *prims = nullptr;  // 40 B triangles or 24 B 2D segments
    const unsigned char *sils = nullptr;   // 56 B edges or 32 B 2D vertices
    uint32_t nNodes = 0, nPrims = 0, nSils = 0, maxDepth = 0;
    uint32_t *errorWord = nullptr;
};

// binary-tree query kernels (k_binary.cu)
cudaError_t launchClosestPointBinary(const SceneView &v, const DevSphere *spheres, DevInteraction *out,
                                     uint32_t n, int recordNormal, cudaStream_t s);
// counting variant: stats[0..2] += popped nodes, expanded inner nodes, primitive tests
cudaError_t launchClosestPointBinaryStats(const SceneView &v, const DevSphere *spheres, DevInteraction *out,
                                          uint32_t n, unsigned long long *stats, cudaStream_t s);
cudaError_t launchRayBinary(const SceneView &v, const DevRay *rays, DevInteraction *out, uint32_t n, int occl,
                            cudaStream_t s);
cudaError_t launchSphereSampleBinary(const SceneView &v, const DevSphere *spheres, const float3 *randNums,
                                     DevInteraction *out, uint32_t n, cudaStream_t s);
// perm: sorted position -> caller query (spheres sorted, flip and out in caller order), or NULL
cudaError_t launchSilhouetteBinary(const SceneView &v, const DevSphere *spheres, const uint32_t *flip,
                                   const uint32_t *perm, DevInteraction *out, uint32_t n, float sqMinR,
                                   float precision, cudaStream_t s);
cudaError_t launchFillDefault(DevInteraction *out, uint32_t n, cudaStream_t s);

// Scene::contains and hasLineOfSight with the reference CPU arithmetic (k_inside.cu);
// points are 3 floats each, results 0 / 1 (contains: 2 when a ray had too many hits)
// points at points[stride * q]; perm non-NULL: points in sorted order, answers to out[perm[q]]
cudaError_t launchContains(const SceneView &v, const float *points, uint32_t stride, const uint32_t *perm,
                           uint32_t n, uint32_t *out, cudaStream_t s);
cudaError_t launchPackPoints(const float *points, uint32_t n, DevSphere *out, cudaStream_t s);
cudaError_t launchLineOfSight(const SceneView &v, const float *a, const float *b, uint32_t n, uint32_t *out,
                              cudaStream_t s);

// FP64 brute-force closest distance of every query over all primitives (k_check.cu)
cudaError_t launchBruteF64(int dim, const unsigned char *prims, uint32_t nPrims, const DevSphere *spheres,
                           uint32_t n, double *out, cudaStream_t s);

// wide / quantised closest point (k_wide.cuh, k_wide_w{2,4,8}.cu)
struct WideLaunch {
    const unsigned char *nodes = nullptr;  // wide node records
    const unsigned char *prims = nullptr;  // 48 B triangles (3D) or 24 B segments (2D)
    const DevSphere *spheres = nullptr;    // queries (sorted when perm is set)
    const uint32_t *perm = nullptr;        // sorted position -> caller query index, or NULL
    const uint32_t *roots = nullptr;       // root record of every (sorted) query in a forest, or NULL (root 0)
    DevInteraction *out = nullptr;
    uint2 *sel = nullptr;                  // precise mode on triangles: per (sorted) query, winner and runner-up leaf positions
    uint32_t n = 0;
    int recordNormal = 0;
    uint32_t *counter = nullptr;           // work counter (zero on entry) for persistent blocks, or NULL
    int packet = 0;                        // 1: warp packets (kWidePacketClosestPoint), counter unused
    int shortStack = 16;                   // per-thread stack entries in shared memory (thread schedules): 0 or 16
    int lanes = 1;                         // > 1: lane groups per query (kWideCoopClosestPoint), counter unused
    uint32_t *errorWord = nullptr;
    unsigned long long *stats = nullptr;   // traversal statistics, or NULL
    uint32_t grid = 0;
    bool deferRefine = false;              // precise mode on triangles: leave the refinement pass to the caller
};
template<int W> cudaError_t launchWideClosestT(int bits, int dim, bool precise, const WideLaunch &l, cudaStream_t s);
// precise mode's second pass on triangles (48 B records): one thread per
// (sorted) query refines the winner and runner-up of sel[i] and writes the
// record to out[perm[i]] (out[i])
cudaError_t launchRefineTriangles(const unsigned char *prims, const DevSphere *spheres, const uint32_t *perm,
                                  const uint2 *sel, DevInteraction *out, uint32_t n, int recordNormal, cudaStream_t s);
// the same pass in the caller's order: thread i refines caller query i
// (spheres in the caller's order) from sel[inv[i]] and writes out[i], so that
// consecutive threads write consecutive records (out may be mapped host memory)
cudaError_t launchRefineTrianglesInOrder(const unsigned char *prims, const DevSphere *spheres, const uint32_t *inv,
                                         const uint2 *sel, DevInteraction *out, uint32_t n, int recordNormal,
                                         cudaStream_t s);
// dispatch over W = 2, 4, 8
cudaError_t launchWide(int W, int bits, int dim, bool precise, const WideLaunch &l, cudaStream_t s);
// closest silhouette points with warp packets on the binary SNCH tree
// (k_sil_packet.cu): queries sorted when perm is set, flip in caller order;
// counter non-NULL (zeroed): grid persistent blocks whose warps take packets from it;
// stats non-NULL (zeroed, 5 words): the counting variant (traversal statistics)
cudaError_t launchSilhouettePacket(const SceneView &v, const DevSphere *spheres, const uint32_t *flip,
                                   const uint32_t *perm, DevInteraction *out, uint32_t n, float sqMinR,
                                   float precision, uint32_t *counter, uint32_t grid, cudaStream_t s,
                                   unsigned long long *stats = nullptr);
// rays on the wide trees (one thread per ray)
struct WideRayLaunch {
    const unsigned char *nodes = nullptr;
    const unsigned char *prims = nullptr;
    const DevRay *rays = nullptr;           // (sorted when perm is set)
    const uint32_t *perm = nullptr;
    const DevRay *callerRays = nullptr;     // with sortInfo: the caller's array, used when keepOrder holds
    const int *sortInfo = nullptr;          // the sort's verdict (cells + kSortCells), or NULL
    DevInteraction *out = nullptr;
    uint32_t n = 0;
    int occl = 0;
    int packet = 0;                         // 1: warp packets (kWidePacketRay)
    uint32_t *counter = nullptr;            // zeroed ray counter: per-lane refill (kWideRayRefill), grid blocks
    uint32_t grid = 0;
    uint32_t *errorWord = nullptr;
    unsigned long long *stats = nullptr;
};
template<int W> cudaError_t launchWideRayT(int bits, int dim, const WideRayLaunch &l, cudaStream_t s);
cudaError_t launchWideRays(int W, int bits, int dim, const WideRayLaunch &l, cudaStream_t s);
template<int W> cudaError_t launchRequantizeT(int bits, unsigned char *wideNodes, const int32_t *childBinary,
                                              const unsigned char *binNodes, int binStride, uint32_t nWide,
                                              uint32_t *errorWord, cudaStream_t s);

// query reordering and record packing (k_sort.cu)
constexpr uint32_t kSortCellBits = 21;  // up to 2^21 cells: 128^3 in 3D (512^2 in 2D)
constexpr uint32_t kSortCells = 1u << kSortCellBits;
// the sort grid spans the query bounds clipped to [lo, hi]
struct SortLimits { float3 lo; float3 hi; int dim; };
// cells: scratch of kSortScratchWords words (counters, query bounds, scan tile sums)
constexpr uint32_t kSortScratchWords = kSortCells + 8 + kSortCells / 4096;
// inv non-NULL: also the inverse permutation, inv[caller index] = sorted position
cudaError_t launchSortQueries(const SortLimits &lim, const DevSphere *spheres, uint32_t n, uint32_t *cells,
                              DevSphere *sorted, uint32_t *perm, int numSMs, cudaStream_t s, uint32_t *inv = nullptr);
// the same for rays: by direction octant, then origin; rays that are already
// coherent keep the caller's order (keepOrder on cells + kSortCells), and with
// skipInOrder then nothing is written to sorted / perm (the caller reads its
// own array)
cudaError_t launchSortRays(const SortLimits &lim, const DevRay *rays, uint32_t n, uint32_t *cells, DevRay *sorted,
                           uint32_t *perm, int numSMs, cudaStream_t s, bool skipInOrder = false);
// exclusive scan of nCells counters in place; tileSums holds batchScanTiles(nCells) words
cudaError_t scanCounts(uint32_t *cells, uint32_t nCells, uint32_t *tileSums, cudaStream_t s);
// stable radix sort of n keys (low keyBits bits) carrying their input index:
// the indices in sorted order end in valsOut (valsAlt: n more words), the
// keys ping-pong between keys0 and keys1 (*sortedKeys: the sorted ones);
// scratch holds radixScratchWords(n) words
size_t radixScratchWords(uint32_t n);
cudaError_t radixSortIndices(uint32_t *keys0, uint32_t *keys1, uint32_t n, int keyBits, uint32_t *valsOut,
                             uint32_t *valsAlt, uint32_t *scratch, const uint32_t **sortedKeys, cudaStream_t s);
cudaError_t launchPackTri48(const DevTriangle *tris, uint32_t n, float4 *out, cudaStream_t s);

// batches of scenes: per-scene sort grid (cells cellBase .. cellBase + 2^(dim*bits))
struct BatchSceneGrid {
    float3 lo, inv;     // grid origin and cells per unit length (2^bits / extent)
    uint32_t cellBase;  // first cell of the scene in the concatenated cell array
    uint32_t bits;      // cells per axis = 2^bits (<= 8 in 3D, <= 12 in 2D)
    uint32_t root;      // wide record of the scene's root in the forest
    uint32_t pad;
};
uint32_t batchScanTiles(uint32_t nCells);  // entries of the tileSums scratch
cudaError_t launchSortBatchQueries(int dim, const BatchSceneGrid *grids, const uint32_t *offsets, uint32_t nScenes,
                                   const DevSphere *spheres, uint32_t n, uint32_t *cells, uint32_t nCells,
                                   uint32_t *tileSums, DevSphere *sorted, uint32_t *perm, uint32_t *roots,
                                   cudaStream_t s);

// the reference's binned SAH tree built on the device (k_sah_build.cu); heuristic
// 0..4 = longest axis, surface area, overlap surface area, volume, overlap volume
struct DeviceBuffer;
int buildSahTree(int dim, int heuristic, const float *positions, const int32_t *indices, uint32_t n,
                 uint32_t *errorWord, cudaStream_t st, DeviceBuffer &nodesOut, DeviceBuffer &primsOut,
                 DeviceBuffer &vertsOut, uint32_t &nNodes);

// GPU BVH construction (k_build.cu)
size_t lbvhScratchWords(uint32_t n);
cudaError_t launchCheckIndices(const int32_t *indices, size_t nIdx, uint32_t nVertices, uint32_t *bad, int numSMs,
                               cudaStream_t s);
// nodesOut: room for 2n - 1 interop nodes; primsOut: n interop primitives;
// primVertsOut: n * dim vertex indices; counters: 8 words ([0] leaves, [1] depth)
cudaError_t launchBuildLbvh(const float *positions, const int32_t *indices, int dim, uint32_t n, uint32_t maxLeaf,
                            uint32_t *scratch, unsigned char *nodesOut, unsigned char *primsOut,
                            int32_t *primVertsOut, uint32_t *counters, uint32_t *errorWord, int numSMs,
                            cudaStream_t s);

// backward of the differentiable queries (k_grad.cu)
struct GradView {
    int dim = 3;
    uint32_t nPrims = 0, nVertices = 0;
    const int32_t *origVerts = nullptr;   // caller vertex of every corner, original primitive order
    const uint32_t *csrOff = nullptr;     // vertex -> corners (nVertices + 1 offsets)
    const uint32_t *csrCorner = nullptr;  // corner ids (prim * dim + corner) in fixed order
    long long *corners = nullptr;         // scratch: nPrims * dim * 3 fixed-point partial sums
    unsigned int *maxBits = nullptr;      // scratch: max |dL/dout| as float bits
};
cudaError_t launchDistanceBackward(const GradView &gv, const DevSphere *spheres, const DevInteraction *fwd,
                                   const float *gradD, uint32_t n, float *gradX, float *gradV, cudaStream_t s);
cudaError_t launchRayBackward(const GradView &gv, const DevRay *rays, const DevInteraction *fwd, const float *gradT,
                              uint32_t n, float *gradO, float *gradDir, float *gradV, cudaStream_t s);

// refit (k_refit.cu)
struct RefitView {
    int dim = 3;
    bool snch = false;
    unsigned char *nodes = nullptr;      // mutable node records
    const unsigned char *prims = nullptr;
    const unsigned char *sils = nullptr;
    const int32_t *parents = nullptr;    // parent node of every node, -1 for the root
    const uint32_t *leaves = nullptr;    // node index of every leaf
    uint32_t nLeaves = 0, nNodes = 0;
    uint32_t *counters = nullptr;        // scratch: one arrival counter per node, zero on entry
};
cudaError_t launchRefit(const RefitView &v, cudaStream_t s);

// device-side geometry regather from caller-order vertex positions (k_refit.cu)
cudaError_t launchGatherPrimitives(int dim, const float *positions, const int32_t *primVerts, uint32_t nPrims,
                                   unsigned char *prims, cudaStream_t s);
cudaError_t launchGatherSilhouettes(int dim, const float *positions, const int32_t *silVerts, uint32_t nSils,
                                    unsigned char *sils, cudaStream_t s);

}  // namespace fcpwgb
