// Precise mode's refinement pass on triangles. The traversal kernels leave,
// per sorted query, the leaf positions of the winner and of the runner-up
// within the rounding band; this pass computes their distances in
// double-single arithmetic (FP64 where ill-conditioned, Tri48Prim::refine),
// keeps the closer one and writes the record to the caller's slot. One
// thread per query in sorted order, so neighbouring threads read
// neighbouring primitives. (Segments refine inside the traversal kernels.)
#include "k_wide.cuh"

namespace fcpwgb {

namespace {

constexpr int kRefineBlock = 256;

// 3 blocks per SM (80 registers; the few spilled bytes sit around the FP64
// fallback call): 0.05 ms faster on 4M queries than 2 blocks at 97 registers
template<class Prim>
__global__ void __launch_bounds__(kRefineBlock, 3) kRefineClosest(const unsigned char *__restrict__ prims,
                                                               const DevSphere *__restrict__ spheres,
                                                               const uint32_t *__restrict__ perm,
                                                               const uint2 *__restrict__ sel,
                                                               DevInteraction *__restrict__ out, uint32_t n,
                                                               int recordNormal) {
    const uint32_t i = blockIdx.x * kRefineBlock + threadIdx.x;
    if (i < n) refineQuery<Prim>(prims, spheres, perm, sel, out, i, recordNormal);
}

}  // namespace

cudaError_t launchRefineTriangles(const unsigned char *prims, const DevSphere *spheres, const uint32_t *perm,
                                  const uint2 *sel, DevInteraction *out, uint32_t n, int recordNormal, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t g = (n + kRefineBlock - 1) / kRefineBlock;
    kRefineClosest<Tri48Prim><<<g, kRefineBlock, 0, s>>>(prims, spheres, perm, sel, out, n, recordNormal);
    return cudaGetLastError();
}

}  // namespace fcpwgb
