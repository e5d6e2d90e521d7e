// Host-side state of one GPU scene (the object behind fcpwgb_gpu_scene *).
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "fcpw_gb300.h"
#include "kernels.h"
#include "wide.h"

namespace fcpwgb {

int setError(int code, const std::string &msg);
int cudaFail(cudaError_t e, const char *where);
// Device arrays of queries and records must start on the boundaries the
// kernels read them on: a sphere is one 16 B vector, rays and interaction
// records are read and written in 8 B parts (cudaMalloc and torch
// allocations, and every element of them, satisfy this). Returns
// FCPWGB_ERR_INVALID_ARGUMENT otherwise, before anything is launched.
int checkAligned(const void *p, size_t bytes, const char *what);
// consumes one injected allocation failure (fcpwgb_debug_fail_allocations)
bool injectedAllocFailure();

// Grow-only device allocation owned by a scene.
struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    ~DeviceBuffer() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    int ensure(size_t n) {
        if (n <= bytes) return 0;
        if (injectedAllocFailure())
            return setError(FCPWGB_ERR_OUT_OF_MEMORY, "cudaMalloc: injected allocation failure");
        release();
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e != cudaSuccess) {
            ptr = nullptr;
            cudaGetLastError();
            return cudaFail(e, "cudaMalloc");
        }
        bytes = n;
        return 0;
    }
    int upload(const void *src, size_t n, cudaStream_t s) {
        int rc = ensure(n > 0 ? n : 16);
        if (rc) return rc;
        if (n == 0) return 0;
        cudaError_t e = cudaMemcpyAsync(ptr, src, n, cudaMemcpyHostToDevice, s);
        return e == cudaSuccess ? 0 : cudaFail(e, "cudaMemcpyAsync");
    }
};

struct InstancedState;  // several objects / instances (instanced.cu)

struct GpuScene {
    int dim = 3;
    int device = 0;
    cudaStream_t stream = nullptr;

    // transferred binary tree
    bool transferred = false;
    int bvhType = 0;
    bool snch = false;
    uint32_t nNodes = 0, nPrims = 0, nSils = 0, nLeaves = 0, maxDepth = 0, nVertices = 0;
    uint64_t treeVersion = 0;
    DeviceBuffer nodes, prims, sils, parents, leaves, counters, primVerts, silVerts, errorWord;

    // host copy of the transferred topology (input of the wide collapse)
    std::vector<uint32_t> hostNP, hostOff;
    std::vector<float> hostBoxes;  // pMin[3], pMax[3] per node, as transferred
    float rootBox[6] = {0, 0, 0, 0, 0, 0};

    // derived wide / quantised tree (built on demand, see wide.h)
    WideConfig wideConfig;
    WideTree wide;
    DeviceBuffer wideNodes, wideChildBinary, widePrims;
    // scratch of the fast path: query sort cells / permutation / sorted copy, work counter,
    // precise mode's winner and runner-up leaf positions
    DeviceBuffer sortCells, sortPerm, sortInv, sortSpheres, sortRays, workCounter, refineSel, packedPoints;
    int numSMs = 0;

    // optional event timing of traversal launches
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timedEvents, freeEvents;
    int timeStart(cudaStream_t st);
    int timeEnd(cudaStream_t st);
    ~GpuScene() {
        for (auto &p : timedEvents) { cudaEventDestroy(p.first); cudaEventDestroy(p.second); }
        for (auto &p : freeEvents) { cudaEventDestroy(p.first); cudaEventDestroy(p.second); }
    }

    bool hasTopology = false;  // prim_vertices were given at transfer (device updates, gradients)
    // device address of the static refit scratch (static_scratch.cu), resolved when the tree is
    // transferred; NULL when that failed (staticScratchError says why)
    uint32_t *staticCounters = nullptr;
    std::string staticScratchError;
    // differentiation: corner -> caller vertex table and the static vertex -> corner CSR
    DeviceBuffer origVerts, csrOff, csrCorner, gradCorners, gradMax;

    // staging for the host-array entry points
    DeviceBuffer qIn0, qIn1, qOut;

    int activate() const;
    SceneView view() const;
    cudaStream_t pick(void *s) const;
    // wide trees read from a scene file: (leaf size, tree), used instead of the host collapse
    std::vector<std::pair<int, WideHost>> preloadedWide;
    void resetTree() {
        transferred = false;
        wide.clear();
        preloadedWide.clear();
        inst.reset();
    }
    // set by fcpwgb_gpu_scene_transfer_instanced instead of a single tree
    std::shared_ptr<InstancedState> inst;

    // query dispatch (variant chosen by wideConfig)
    int closestPoints(const DevSphere *spheres, DevInteraction *out, uint32_t n, int recordNormal, cudaStream_t st);
    int closestPointsStats(const DevSphere *spheres, DevInteraction *out, uint32_t n, unsigned long long *stats,
                           cudaStream_t st);
    int rays(const DevRay *rays, DevInteraction *out, uint32_t n, int occl, cudaStream_t st);
    // contains: points sorted spatially first with a fast-path configuration
    int containsPoints(const float *points, uint32_t n, uint32_t *result, cudaStream_t st);
    int closestPointsHost(const fcpwgb_bounding_sphere *spheres, fcpwgb_interaction *out, uint32_t n,
                          int recordNormal);
    // keeps derived trees in step after the binary tree was refit on stream st
    int afterRefit(cudaStream_t st);
    // builds (or rebuilds) the wide tree the current config asks for
    int ensureWide(cudaStream_t st);
    bool useWide() const { return wideConfig.branching > 0; }
    // silhouette queries as warp packets (with a fast-path configuration and no
    // positive minimum radius, whose early stop follows the reference's
    // visiting order)
    bool usePacketSilhouettes(float sqMinR) const { return useWide() && !(sqMinR > 0.0f); }
    int wideRays(const DevRay *rays, DevInteraction *out, uint32_t n, int occl, cudaStream_t st);
    SortLimits sortLimits() const;
    int smCount();  // multiprocessors of the scene's device (queried once)
    // inv non-NULL (n words), with the queries sorted: the sort also writes the
    // inverse permutation there and precise mode on triangles stops after the
    // traversal, leaving sel for the caller's refinement pass
    int wideClosest(const DevSphere *spheres, DevInteraction *out, uint32_t n, int recordNormal,
                    unsigned long long *stats, cudaStream_t st, uint32_t *inv = nullptr);
};

}  // namespace fcpwgb

struct fcpwgb_gpu_scene : fcpwgb::GpuScene {};

namespace fcpwgb {
int runRefit(fcpwgb_gpu_scene *s, cudaStream_t st);
// the checks every single-tree operation makes first (capi.cu)
int requireTree(fcpwgb_gpu_scene *s);
// resolves the static refit scratch on the scene's (current) device (static_scratch.cu)
void resolveStaticScratch(fcpwgb_gpu_scene *s);
// instanced scenes (instanced.cu); instOut may be NULL
int instancedClosest(fcpwgb_gpu_scene *s, const DevSphere *spheres, DevInteraction *out, uint32_t *instOut,
                     uint32_t n, int recordNormal, cudaStream_t st);
int instancedRays(fcpwgb_gpu_scene *s, const DevRay *rays, DevInteraction *out, uint32_t *instOut, uint32_t n,
                  int occl, cudaStream_t st);
int instancedHost(fcpwgb_gpu_scene *s, const void *queries, size_t queryBytes, void *out, uint32_t *instOut,
                  uint32_t n, bool rays, int flag);
enum class InstancedQuery { Closest, Rays, Sample, Silhouette };
int instancedHostQuery(fcpwgb_gpu_scene *s, InstancedQuery kind, const void *queries, size_t queryBytes,
                       const void *second, size_t secondBytes, void *out, uint32_t *instOut, uint32_t n, int flag,
                       float sqMinR, float precision);
int instancedSilhouettes(fcpwgb_gpu_scene *s, const DevSphere *spheres, const uint32_t *flip, DevInteraction *out,
                         uint32_t *instOut, uint32_t n, float sqMinR, float precision, cudaStream_t st);
int instancedSample(fcpwgb_gpu_scene *s, const DevSphere *spheres, const float3 *randNums, DevInteraction *out,
                    uint32_t *instOut, uint32_t n, cudaStream_t st);
int instancedTopRefit(fcpwgb_gpu_scene *s, cudaStream_t st);
}
