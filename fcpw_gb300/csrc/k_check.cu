// FP64 brute-force closest distances: the accuracy probe that every traversal
// variant's FP32 results are measured against. Each query is one block whose
// threads stride over all primitives, each distance computed in FP64 with the
// primitive taken relative to the query; the block keeps the minimum.
// O(queries x primitives): for samples of a batch, not for whole batches.
#include "k_wide.cuh"

namespace fcpwgb {

namespace {

constexpr int kCheckThreads = 256;

template<int DIM>
__global__ void __launch_bounds__(kCheckThreads) kBruteF64(const unsigned char *__restrict__ prims, uint32_t nPrims,
                                                           const DevSphere *__restrict__ q, uint32_t n,
                                                           double *out) {
    __shared__ double part[kCheckThreads / 32];
    const uint32_t i = blockIdx.x;
    if (i >= n) return;
    float4 s = ldg4(q + i);
    float3 c = make_float3(s.x, s.y, s.z);
    double best = 1.0e300;
    for (uint32_t k = threadIdx.x; k < nPrims; k += kCheckThreads) {
        float3 p;
        double d;
        if (DIM == 3) {
            TriPrim t = TriPrim::load(prims, k);
            Tri48Prim w;
            w.pa = t.pa;
            w.pb = t.pb;
            w.pc = t.pc;
            w.index = t.index;
            d = w.refine64(c, p);
        } else {
            d = Seg24Prim::load(prims, k).refine64(c, p);
        }
        best = fmin(best, d);
    }
    for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kCheckThreads / 32; w++) best = fmin(best, part[w]);
        out[i] = nPrims ? best : __longlong_as_double(0x7ff0000000000000ll);  // +inf without primitives
    }
}

}  // namespace

cudaError_t launchBruteF64(int dim, const unsigned char *prims, uint32_t nPrims, const DevSphere *spheres,
                           uint32_t n, double *out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (dim == 3) kBruteF64<3><<<n, kCheckThreads, 0, s>>>(prims, nPrims, spheres, n, out);
    else kBruteF64<2><<<n, kCheckThreads, 0, s>>>(prims, nPrims, spheres, n, out);
    return cudaGetLastError();
}

}  // namespace fcpwgb
