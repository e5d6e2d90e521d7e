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

// the pass in the caller's order (launchRefineTrianglesInOrder)
template<class Prim>
__global__ void __launch_bounds__(kRefineBlock, 3) kRefineClosestInOrder(const unsigned char *__restrict__ prims,
                                                                      const DevSphere *__restrict__ spheres,
                                                                      const uint32_t *__restrict__ inv,
                                                                      const uint2 *__restrict__ sel,
                                                                      DevInteraction *__restrict__ out, uint32_t n,
                                                                      int recordNormal) {
    // the block's records are staged in shared memory and written as 16 B
    // vectors by consecutive threads, so that every store covers whole lines
    // of out (mapped host memory takes partial lines slowly)
    __shared__ float4 stage[kRefineBlock * sizeof(DevInteraction) / sizeof(float4)];
    const uint32_t base = blockIdx.x * kRefineBlock, i = base + threadIdx.x;
    if (i < n) {
        const uint2 s = __ldg(sel + __ldg(inv + i));
        DevInteraction best = defaultInteraction();
        if (s.x != kUintMax) {
            const float4 s4 = ldg4(spheres + i);
            best = refineCandidates<Prim>(prims, make_float3(s4.x, s4.y, s4.z), s.x, s.y, recordNormal);
        }
        reinterpret_cast<DevInteraction *>(stage)[threadIdx.x] = best;
    }
    __syncthreads();
    const uint32_t count = min(n - base, (uint32_t)kRefineBlock);
    const uint32_t vecs = count * (uint32_t)sizeof(DevInteraction) / (uint32_t)sizeof(float4);  // 40 B records: 2.5 vectors
    float4 *dst = reinterpret_cast<float4 *>(out + base);
    for (uint32_t k = threadIdx.x; k < vecs; k += kRefineBlock) dst[k] = stage[k];
    if ((count & 1u) && threadIdx.x == 0) {  // an odd count leaves the last record's final 8 B
        reinterpret_cast<float2 *>(out + base + count)[-1] = reinterpret_cast<const float2 *>(stage)[count * 5 - 1];
    }
}

}  // namespace

cudaError_t launchRefineTrianglesInOrder(const unsigned char *prims, const DevSphere *spheres, const uint32_t *inv,
                                         const uint2 *sel, DevInteraction *out, uint32_t n, int recordNormal,
                                         cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t g = (n + kRefineBlock - 1) / kRefineBlock;
    kRefineClosestInOrder<Tri48Prim><<<g, kRefineBlock, 0, s>>>(prims, spheres, inv, sel, out, n, recordNormal);
    return cudaGetLastError();
}

cudaError_t launchRefineTriangles(const unsigned char *prims, const DevSphere *spheres, const uint32_t *perm,
                                  const uint2 *sel, DevInteraction *out, uint32_t n, int recordNormal, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t g = (n + kRefineBlock - 1) / kRefineBlock;
    kRefineClosest<Tri48Prim><<<g, kRefineBlock, 0, s>>>(prims, spheres, perm, sel, out, n, recordNormal);
    return cudaGetLastError();
}

}  // namespace fcpwgb
