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
//
// Set-up: the array's device address is resolved with cudaGetSymbolAddress
// when a tree is transferred (fcpwgb_gpu_scene_transfer and every entry point
// that ends in it), with the scene's device current. Resolving it loads this
// file's module, and loading the module is what reserves the 4 MiB, so that
// happens inside the transfer, which allocates anyway, and never inside the
// allocation-free call. The address is kept in the scene beside its other
// device buffers and is as valid as they are: a cudaDeviceReset invalidates
// both, and the scene must then be transferred again.
#include <string>

#include <cuda_runtime.h>

#include "fcpw_gb300.h"
#include "kernels.h"
#include "scene.h"

using namespace fcpwgb;

namespace {

constexpr uint32_t kStaticRefitMaxNodes = 1u << 20;

static __device__ __align__(256) uint32_t g_refitCounters[kStaticRefitMaxNodes];

int cudaCheck(cudaError_t e, const char *where) { return e == cudaSuccess ? FCPWGB_OK : cudaFail(e, where); }

}  // namespace

namespace fcpwgb {
void resolveStaticScratch(fcpwgb_gpu_scene *s) {
    s->staticCounters = nullptr;
    s->staticScratchError.clear();
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_refitCounters);
    if (e != cudaSuccess) {
        cudaGetLastError();
        s->staticScratchError = std::string("cudaGetSymbolAddress(g_refitCounters) failed at transfer: ") +
                                cudaGetErrorString(e);
        return;
    }
    if (!p) {
        s->staticScratchError = "cudaGetSymbolAddress(g_refitCounters) returned NULL at transfer";
        return;
    }
    s->staticCounters = (uint32_t *)p;
}
}  // namespace fcpwgb

extern "C" int fcpwgb_gpu_scene_update_vertices_device_static(fcpwgb_gpu_scene *s, const float *positions,
                                                              uint32_t n_vertices, void *stream) {
    int rc = requireTree(s);  // the same checks, in the same order, as the scene-scratch entry point
    if (rc) return rc;
    if (!s->hasTopology) return setError(FCPWGB_ERR_UNSUPPORTED, "the tree was transferred without prim_vertices");
    if (!positions || n_vertices != s->nVertices)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT, "positions must hold the transferred vertex count");
    if (s->nNodes > kStaticRefitMaxNodes)
        return setError(FCPWGB_ERR_INVALID_ARGUMENT,
                        "tree has " + std::to_string(s->nNodes) + " nodes; the static refit scratch holds at most " +
                            std::to_string(kStaticRefitMaxNodes));
    if (!s->staticCounters) return setError(FCPWGB_ERR_CUDA, s->staticScratchError);
    uint32_t *counters = s->staticCounters;

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

// Testing aid: fills the first n words of the shared static array with `word`
// on the scene's device (a plain memset; nothing is allocated), so that a test
// can check that the allocation-free refit clears the counters it uses.
extern "C" int fcpwgb_debug_fill_static_scratch(fcpwgb_gpu_scene *s, uint32_t word, uint32_t n) {
    int rc = requireTree(s);
    if (rc) return rc;
    if (!s->staticCounters) return setError(FCPWGB_ERR_CUDA, s->staticScratchError);
    if (n > kStaticRefitMaxNodes) n = kStaticRefitMaxNodes;
    std::vector<uint32_t> host(n, word);
    if ((rc = cudaCheck(cudaMemcpy(s->staticCounters, host.data(), (size_t)n * sizeof(uint32_t),
                                   cudaMemcpyHostToDevice),
                        "fill static scratch")))
        return rc;
    return FCPWGB_OK;
}
