// Backward kernels of the differentiable queries.
//
// Both read the forward interaction record (p, n, uv, d, index) so nothing is
// traversed again:
//   unsigned distance d(x) = |x - p|, p = sum_k b_k v_k on the closest primitive:
//       dd/dx = (x - p) / d,   dd/dv_k = -b_k (x - p) / d
//   ray hit distance t with the hit on the plane n.(o + t dir - p) = 0:
//       dt/do = -n / (n.dir),  dt/ddir = -t n / (n.dir),  dt/dv_k = b_k n / (n.dir)
// with the barycentric weights b_k recovered from the record's uv (triangles:
// uv = (b_a, b_b); segments: uv.x = weight of the second vertex).
//
// Vertex gradients are reduced deterministically in two stages: every query
// adds its per-corner contributions to its primitive's corners as 64-bit
// fixed-point integers (integer addition is associative, so the totals do not
// depend on arrival order), then each vertex sums its incident corners over a
// static CSR in a fixed order and converts once to float. The fixed-point
// scale is 2^s with s chosen from max|dL/dout| and the query count so that no
// partial sum can overflow.
#include "kernels.h"

namespace fcpwgb {

FCPWGB_D void baryWeights(int dim, float2 uv, float b[3]) {
    if (dim == 3) {
        b[0] = uv.x;
        b[1] = uv.y;
        b[2] = 1.0f - uv.x - uv.y;
    } else {
        b[0] = 1.0f - uv.x;
        b[1] = uv.x;
        b[2] = 0.0f;
    }
}

// max |g| over the batch (order independent)
__global__ void kAbsMax(const float *g, uint32_t n, unsigned int *out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float v = i < n ? fabsf(g[i]) : 0.0f;
    if (!(v == v)) v = 0.0f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(v));  // non-negative floats order like uints
}

FCPWGB_D double fixedScale(unsigned int maxBits, uint32_t n) {
    float m = __uint_as_float(maxBits);
    int eg = m > 0.0f ? ilogbf(m) + 1 : 0;  // |g| < 2^eg
    int en = 32 - __clz(n > 0 ? n : 1);     // n < 2^en
    int s = 60 - eg - en;                   // sum of <= n terms below 2^(60 - en) each stays < 2^60
    if (s > 1000) s = 1000;
    return exp2((double)s);
}

FCPWGB_D void addFixed(long long *acc, float v, double scale) {
    long long q = __double2ll_rn((double)v * scale);
    if (q != 0) atomicAdd(reinterpret_cast<unsigned long long *>(acc), (unsigned long long)q);
}

__global__ void kDistanceGrad(int dim, const DevSphere *__restrict__ spheres,
                              const DevInteraction *__restrict__ fwd, const float *__restrict__ gradD, uint32_t n,
                              const int32_t *__restrict__ origVerts, uint32_t nPrims, float *gradX,
                              long long *corners, const unsigned int *maxBits) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    DevInteraction r = fwd[q];
    float3 x = make_float3(spheres[q].c.x, spheres[q].c.y, spheres[q].c.z);
    float g = gradD[q];
    // u = (x - p) / |x - p|: the unit gradient of the distance, normalised by the
    // length of the difference actually formed so that |u| = 1 to rounding
    float3 u = make_float3(0.f, 0.f, 0.f);
    float3 diff = x - r.p;
    float len = len3(diff);
    bool valid = r.index < nPrims && r.d > 0.0f && len > 0.0f && g == g;
    if (valid) u = diff / len;
    gradX[dim * q] = valid ? g * u.x : 0.0f;
    gradX[dim * q + 1] = valid ? g * u.y : 0.0f;
    if (dim == 3) gradX[dim * q + 2] = valid ? g * u.z : 0.0f;
    if (!valid) return;
    double scale = fixedScale(*maxBits, n);
    float b[3];
    baryWeights(dim, r.uv, b);
    for (int k = 0; k < dim; k++) {
        long long *c = corners + 3ull * ((size_t)r.index * dim + k);
        float w = -g * b[k];
        addFixed(c, w * u.x, scale);
        addFixed(c + 1, w * u.y, scale);
        if (dim == 3) addFixed(c + 2, w * u.z, scale);
    }
}

__global__ void kRayGrad(int dim, const DevRay *__restrict__ rays, const DevInteraction *__restrict__ fwd,
                         const float *__restrict__ gradT, uint32_t n, uint32_t nPrims, float *gradO, float *gradDir,
                         long long *corners, const unsigned int *maxBits) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    DevInteraction r = fwd[q];
    DevRay ray = rays[q];
    float g = gradT[q];
    float nd = dot3(r.n, ray.d);
    bool valid = r.index < nPrims && r.d < kFltMax && fabsf(nd) > 0.0f && g == g;
    float3 k = valid ? r.n * (g / nd) : make_float3(0.f, 0.f, 0.f);  // g n / (n.dir)
    float3 go = make_float3(-k.x, -k.y, -k.z), gd = make_float3(-k.x * r.d, -k.y * r.d, -k.z * r.d);
    gradO[dim * q] = go.x;
    gradO[dim * q + 1] = go.y;
    gradDir[dim * q] = gd.x;
    gradDir[dim * q + 1] = gd.y;
    if (dim == 3) {
        gradO[dim * q + 2] = go.z;
        gradDir[dim * q + 2] = gd.z;
    }
    if (!valid) return;
    double scale = fixedScale(*maxBits, n);
    float b[3];
    baryWeights(dim, r.uv, b);
    for (int c = 0; c < dim; c++) {
        long long *acc = corners + 3ull * ((size_t)r.index * dim + c);
        addFixed(acc, b[c] * k.x, scale);
        addFixed(acc + 1, b[c] * k.y, scale);
        if (dim == 3) addFixed(acc + 2, b[c] * k.z, scale);
    }
}

// per vertex: fixed-order sum over its corners (static CSR), then one conversion
__global__ void kVertexGrad(int dim, const uint32_t *__restrict__ csrOff, const uint32_t *__restrict__ csrCorner,
                            uint32_t nVertices, const long long *__restrict__ corners, const unsigned int *maxBits,
                            uint32_t n, float *gradV) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nVertices) return;
    long long s0 = 0, s1 = 0, s2 = 0;
    for (uint32_t i = csrOff[v]; i < csrOff[v + 1]; i++) {
        const long long *c = corners + 3ull * csrCorner[i];
        s0 += c[0];
        s1 += c[1];
        s2 += c[2];
    }
    double inv = 1.0 / fixedScale(*maxBits, n);
    gradV[dim * v] = (float)((double)s0 * inv);
    gradV[dim * v + 1] = (float)((double)s1 * inv);
    if (dim == 3) gradV[dim * v + 2] = (float)((double)s2 * inv);
}

cudaError_t launchDistanceBackward(const GradView &gv, const DevSphere *spheres, const DevInteraction *fwd,
                                   const float *gradD, uint32_t n, float *gradX, float *gradV, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(gv.maxBits, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(gv.corners, 0, (size_t)gv.nPrims * gv.dim * 3 * sizeof(long long), s);
    if (e != cudaSuccess) return e;
    uint32_t blocks = (n + 255) / 256;
    if (n > 0) {
        kAbsMax<<<blocks, 256, 0, s>>>(gradD, n, gv.maxBits);
        kDistanceGrad<<<blocks, 256, 0, s>>>(gv.dim, spheres, fwd, gradD, n, gv.origVerts, gv.nPrims, gradX,
                                             gv.corners, gv.maxBits);
    }
    if (gv.nVertices > 0)
        kVertexGrad<<<(gv.nVertices + 255) / 256, 256, 0, s>>>(gv.dim, gv.csrOff, gv.csrCorner, gv.nVertices,
                                                              gv.corners, gv.maxBits, n, gradV);
    return cudaGetLastError();
}

cudaError_t launchRayBackward(const GradView &gv, const DevRay *rays, const DevInteraction *fwd, const float *gradT,
                              uint32_t n, float *gradO, float *gradDir, float *gradV, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(gv.maxBits, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(gv.corners, 0, (size_t)gv.nPrims * gv.dim * 3 * sizeof(long long), s);
    if (e != cudaSuccess) return e;
    uint32_t blocks = (n + 255) / 256;
    if (n > 0) {
        kAbsMax<<<blocks, 256, 0, s>>>(gradT, n, gv.maxBits);
        kRayGrad<<<blocks, 256, 0, s>>>(gv.dim, rays, fwd, gradT, n, gv.nPrims, gradO, gradDir, gv.corners,
                                        gv.maxBits);
    }
    if (gv.nVertices > 0)
        kVertexGrad<<<(gv.nVertices + 255) / 256, 256, 0, s>>>(gv.dim, gv.csrOff, gv.csrCorner, gv.nVertices,
                                                              gv.corners, gv.maxBits, n, gradV);
    return cudaGetLastError();
}

}  // namespace fcpwgb
