// Device vertex update + refit whose scratch lives in a file-scope device
// array instead of memory the scene allocates: for callers that may not call
// cudaMalloc while they run. The bottom-up refit needs one arrival counter per
// node (k_refit.cu); here those counters come from g_refitCounters.
//
// g_refitCounters is a static __device__ array of kStaticRefitMaxNodes 32-bit
// words (4 MiB). Every GPU that loads this library holds it until the process
// exits. All calls on a device share it and it keeps the previous call's
// contents, so each call clears the counters it uses before the refit kernel
// runs; two calls whose work overlaps on the GPU (different streams, scenes or
// threads) race on the counters and must be ordered by the caller.
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "fcpw_gb300.h"
#include "kernels.h"
#include "scene.h"

using namespace fcpwgb;

namespace {

constexpr uint32_t kStaticRefitMaxNodes = 1u << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint32_t g_refitCounters[kStaticRefitMaxNodes];

std::mutex g_setupMutex;
uint32_t *g_countersOnDevice[kMaxDevices] = {};

// Resolves g_refitCounters on `device`, which must be the current device.
// Runs once per device; later calls return the cached address.
int counterAddress(int device, uint32_t **out) {
    if (device < 0 || device >= kMaxDevices)
        return setError(FCPWGB_ERR_UNSUPPORTED, "device ordinal beyond the static scratch table (64 devices)");
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_countersOnDevice[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_refitCounters);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cudaFail(e, "cudaGetSymbolAddress(g_refitCounters)");
        }
        if (!p) return setError(FCPWGB_ERR_CUDA, "cudaGetSymbolAddress(g_refitCounters) returned NULL");
        g_countersOnDevice[device] = (uint32_t *)p;
    }
    *out = g_countersOnDevice[device];
    return FCPWGB_OK;
}

int cudaCheck(cudaError_t e, const char *where) { return e == cudaSuccess ? FCPWGB_OK : cudaFail(e, where); }

}  // namespace

extern "C" int fcpwgb_gpu_scene_update_vertices_device_static(fcpwgb_gpu_scene *s, const float *positions,
                                                              uint32_t n_vertices, void *stream) {
    if (!s) return setError(FCPWGB_ERR_INVALID_ARGUMENT, "NULL scene");
    if (!s->transferred) return setError(FCPWGB_ERR_NOT_TRANSFERRED, "transferToGPU has not been called");
    if (s->nNodes > kStaticRefitMaxNodes)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT,
                        "tree has " + std::to_string(s->nNodes) + " nodes; the static refit scratch holds at most " +
                            std::to_string(kStaticRefitMaxNodes));
    if (!s->hasTopology) return setError(FCPWGB_ERR_UNSUPPORTED, "the tree was transferred without prim_vertices");
    if (!positions || n_vertices != s->nVertices)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "positions must hold the transferred vertex count");
    int rc = s->activate();
    if (rc) return rc;
    uint32_t *counters = nullptr;
    if ((rc = counterAddress(s->device, &counters))) return rc;

    cudaStream_t st = s->pick(stream);
    if ((rc = cudaCheck(launchGatherPrimitives(s->dim, positions, (const int32_t *)s->primVerts.ptr, s->nPrims,
                                               (unsigned char *)s->prims.ptr, st),
                        "gather primitives")))
        return rc;
    if (s->snch && s->nSils > 0 && s->silVerts.ptr &&
        (rc = cudaCheck(launchGatherSilhouettes(s->dim, positions, (const int32_t *)s->silVerts.ptr, s->nSils,
                                                (unsigned char *)s->sils.ptr, st),
                        "gather silhouettes")))
        return rc;
    // the array still holds the previous call's arrivals
    if ((rc = cudaCheck(cudaMemsetAsync(counters, 0, (size_t)s->nNodes * sizeof(uint32_t), st), "clear counters")))
        return rc;
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
    v.counters = counters;
    if ((rc = cudaCheck(launchRefit(v, st), "refit"))) return rc;
    return s->afterRefit(st);
}
