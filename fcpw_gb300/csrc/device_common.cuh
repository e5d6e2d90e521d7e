// Device-side records, loads and geometric primitives shared by the query kernels.
//
// Device layouts (chosen at transfer time, see capi.cu):
//   binary node  : 32 B, byte-identical to GPUBvhNode {pMin, pMax, nPrimitives, offset}
//   SNCH node    : 64 B, the same 32 B prefix followed by {axis, halfAngle, radius,
//                  nSilhouettes, silhouetteOffset, pad}
//   triangle     : 40 B, byte-identical to GPUTriangle {pa, pb, pc, index}
//   segment (2D) : 24 B {pa.xy, pb.xy, index, pad}
//   edge (3D)    : 56 B, byte-identical to GPUEdge
//   vertex (2D)  : 32 B {p.xy, n0.xy, n1.xy, index, hasOneAdjacentFace}
// All arrays come from cudaMalloc (256 B aligned), so the 16 B and 8 B vector
// loads below are aligned for every element.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fcpwgb {

#define FCPWGB_HD __host__ __device__ __forceinline__
#define FCPWGB_D __device__ __forceinline__

constexpr float kFltMax = 3.402823466e+38F;
constexpr float kFltEps = 1.192092896e-07F;
constexpr float kPiF = 3.14159265358979323846f;
constexpr float kPi2F = 1.57079632679489661923f;
constexpr uint32_t kUintMax = 0xffffffffu;
constexpr int kStackDepth = 64;  // FCPW_BVH_MAX_DEPTH

// device error word bits
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrStepBudget = 2u;
constexpr uint32_t kErrBadIndex = 4u;

struct DevInteraction {  // 40 B, GPUInteraction
    float3 p;
    float3 n;
    float2 uv;
    float d;
    uint32_t index;
};
static_assert(sizeof(DevInteraction) == 40, "GPUInteraction layout");

struct DevRay { float3 o, d, dInv; float tMax; };
static_assert(sizeof(DevRay) == 40, "GPURay layout");
struct DevSphere { float3 c; float r2; };
static_assert(sizeof(DevSphere) == 16, "GPUBoundingSphere layout");

struct DevTriangle { float3 pa, pb, pc; uint32_t index; };
static_assert(sizeof(DevTriangle) == 40, "GPUTriangle layout");
struct DevSegment2 { float2 pa, pb; uint32_t index, pad; };
static_assert(sizeof(DevSegment2) == 24, "segment layout");
struct DevEdge { float3 pa, pb, n0, n1; uint32_t index, hasOneAdjacentFace; };
static_assert(sizeof(DevEdge) == 56, "GPUEdge layout");
struct DevVertex2 { float2 p, n0, n1; uint32_t index, hasOneAdjacentFace; };
static_assert(sizeof(DevVertex2) == 32, "vertex layout");

FCPWGB_HD DevInteraction defaultInteraction() {
    DevInteraction i;
    i.p = make_float3(0.f, 0.f, 0.f);
    i.n = make_float3(0.f, 0.f, 0.f);
    i.uv = make_float2(0.f, 0.f);
    i.d = kFltMax;
    i.index = kUintMax;
    return i;
}

// --------------------------------------------------------------- float3 ops
FCPWGB_HD float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
FCPWGB_HD float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
FCPWGB_HD float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
FCPWGB_HD float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }
FCPWGB_HD float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
FCPWGB_HD float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
FCPWGB_HD float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
FCPWGB_HD float len3(float3 a) { return sqrtf(dot3(a, a)); }
FCPWGB_HD float3 normalize3(float3 a) {
    float z = dot3(a, a);
    return z > 0.0f ? a / sqrtf(z) : a;
}
FCPWGB_HD float3 fmin3(float3 a, float3 b) { return make_float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
FCPWGB_HD float3 fmax3(float3 a, float3 b) { return make_float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }

// --------------------------------------------------------------- loads
FCPWGB_D float4 ldg4(const void *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
FCPWGB_D float2 ldg2(const void *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }

// binary / SNCH node prefix: box + nPrimitives + offset
struct NodeBox {
    float3 pMin, pMax;
    uint32_t nPrims, offset;
};
template<int STRIDE_BYTES>
FCPWGB_D NodeBox loadNode(const unsigned char *nodes, uint32_t i) {
    const unsigned char *p = nodes + (size_t)i * STRIDE_BYTES;
    float4 a = ldg4(p), b = ldg4(p + 16);
    NodeBox n;
    n.pMin = make_float3(a.x, a.y, a.z);
    n.pMax = make_float3(a.w, b.x, b.y);
    n.nPrims = __float_as_uint(b.z);
    n.offset = __float_as_uint(b.w);
    return n;
}
// The query sort's verdict on a batch of rays (k_sort.cu): sortInfo[6] counts
// how many of up to kCoherenceSamples evenly spaced consecutive pairs point
// alike; with 90 % of them alike the rays are already coherent (camera rays)
// and keep the caller's order.
constexpr uint32_t kCoherenceSamples = 16384;
FCPWGB_D bool keepOrder(const int *sortInfo, uint32_t n) {
    const uint32_t samples = min(n > 0 ? n - 1 : 0u, kCoherenceSamples);
    return samples > 0 && (uint32_t)__ldg(sortInfo + 6) * 10u >= samples * 9u;
}

// SNCH node suffix (bytes 32..63)
struct NodeCone { float3 axis; float halfAngle, radius; uint32_t nSil, silOffset; };
FCPWGB_D NodeCone loadCone(const unsigned char *nodes, uint32_t i) {
    const unsigned char *p = nodes + (size_t)i * 64 + 32;
    float4 a = ldg4(p), b = ldg4(p + 16);
    NodeCone c;
    c.axis = make_float3(a.x, a.y, a.z);
    c.halfAngle = a.w;
    c.radius = b.x;
    c.nSil = __float_as_uint(b.y);
    c.silOffset = __float_as_uint(b.z);
    return c;
}

// sphere-box distances, bounding-volumes.slang:43-64
FCPWGB_HD void boxSphereDist(float3 pMin, float3 pMax, float3 c, float &d2Min, float &d2Max) {
    float3 u = pMin - c, v = c - pMax;
    float ax = fmaxf(fmaxf(u.x, v.x), 0.f), ay = fmaxf(fmaxf(u.y, v.y), 0.f), az = fmaxf(fmaxf(u.z, v.z), 0.f);
    float bx = fminf(u.x, v.x), by = fminf(u.y, v.y), bz = fminf(u.z, v.z);
    d2Min = ax * ax + ay * ay + az * az;
    d2Max = bx * bx + by * by + bz * bz;
}
FCPWGB_HD float boxSphereD2Min(float3 pMin, float3 pMax, float3 c) {
    float3 u = pMin - c, v = c - pMax;
    float ax = fmaxf(fmaxf(u.x, v.x), 0.f), ay = fmaxf(fmaxf(u.y, v.y), 0.f), az = fmaxf(fmaxf(u.z, v.z), 0.f);
    return ax * ax + ay * ay + az * az;
}

// ray-box slab test with the parallel-slab guard, bounding-volumes.slang:67-106
FCPWGB_HD bool boxRayIntersect(float3 pMin, float3 pMax, const DevRay &r, float &tMin, float &tMax) {
    float3 t0 = make_float3((pMin.x - r.o.x) * r.dInv.x, (pMin.y - r.o.y) * r.dInv.y, (pMin.z - r.o.z) * r.dInv.z);
    float3 t1 = make_float3((pMax.x - r.o.x) * r.dInv.x, (pMax.y - r.o.y) * r.dInv.y, (pMax.z - r.o.z) * r.dInv.z);
    float3 tNear = fmin3(t0, t1), tFar = fmax3(t0, t1);
    bool px = r.d.x == 0.0f, py = r.d.y == 0.0f, pz = r.d.z == 0.0f;
    bool wx = r.o.x >= pMin.x && r.o.x <= pMax.x;
    bool wy = r.o.y >= pMin.y && r.o.y <= pMax.y;
    bool wz = r.o.z >= pMin.z && r.o.z <= pMax.z;
    if ((px && !wx) || (py && !wy) || (pz && !wz)) {
        tMin = kFltMax;
        tMax = kFltMax;
        return false;
    }
    if (px) { tNear.x = -kFltMax; tFar.x = kFltMax; }
    if (py) { tNear.y = -kFltMax; tFar.y = kFltMax; }
    if (pz) { tNear.z = -kFltMax; tFar.z = kFltMax; }
    float tNearMax = fmaxf(0.0f, fmaxf(tNear.x, fmaxf(tNear.y, tNear.z)));
    float tFarMin = fminf(r.tMax, fminf(tFar.x, fminf(tFar.y, tFar.z)));
    if (tNearMax > tFarMin) {
        tMin = kFltMax;
        tMax = kFltMax;
        return false;
    }
    tMin = tNearMax;
    tMax = tFarMin;
    return true;
}

}  // namespace fcpwgb
#include "exact_ops.cuh"
namespace fcpwgb {

// ----------------------------------------------------------- primitives

// Ericson's closest point on a triangle (Real-Time Collision Detection,
// section 5.1.5), the region test of geometry.slang:251-332 / triangles.inl:374-458
FCPWGB_HD float closestPointTriangle(float3 pa, float3 pb, float3 pc, float3 x, float3 &p, float2 &t) {
    float3 ab = pb - pa, ac = pc - pa, ax = x - pa;
    float d1 = dot3(ab, ax), d2 = dot3(ac, ax);
    if (d1 <= 0.0f && d2 <= 0.0f) { t = make_float2(1.0f, 0.0f); p = pa; return len3(x - p); }
    float3 bx = x - pb;
    float d3 = dot3(ab, bx), d4 = dot3(ac, bx);
    if (d3 >= 0.0f && d4 <= d3) { t = make_float2(0.0f, 1.0f); p = pb; return len3(x - p); }
    float3 cx = x - pc;
    float d5 = dot3(ab, cx), d6 = dot3(ac, cx);
    if (d6 >= 0.0f && d5 <= d6) { t = make_float2(0.0f, 0.0f); p = pc; return len3(x - p); }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = d1 / (d1 - d3);
        t = make_float2(1.0f - v, v);
        p = pa + ab * v;
        return len3(x - p);
    }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float w = d2 / (d2 - d6);
        t = make_float2(1.0f - w, 0.0f);
        p = pa + ac * w;
        return len3(x - p);
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        t = make_float2(0.0f, 1.0f - w);
        p = pb + (pc - pb) * w;
        return len3(x - p);
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    t = make_float2(1.0f - v - w, v);
    p = pa + ab * v + ac * w;
    return len3(x - p);
}

// closest point on a segment, geometry.slang:79-103
FCPWGB_HD float closestPointSegment(float3 pa, float3 pb, float3 x, float3 &p, float &t) {
    float3 u = pb - pa, v = x - pa;
    float c1 = dot3(u, v);
    if (c1 <= 0.0f) { t = 0.0f; p = pa; return len3(x - p); }
    float c2 = dot3(u, u);
    if (c2 <= c1) { t = 1.0f; p = pb; return len3(x - p); }
    t = c1 / c2;
    p = pa + u * t;
    return len3(x - p);
}

// Ray-primitive tests: the reference's Moller-Trumbore and segment test in its
// own float arithmetic (exact_ops.cuh), so hit distances, points, normals and
// uvs equal the reference's bit for bit
FCPWGB_D bool intersectTriangle(float3 pa, float3 pb, float3 pc, const DevRay &r, bool occl, DevInteraction &i) {
    return xIntersectTriangle(pa, pb, pc, r, occl, i);
}
FCPWGB_D bool intersectSegment(float3 pa, float3 pb, const DevRay &r, bool occl, DevInteraction &i) {
    return xIntersectSegment(pa, pb, r, occl, i);
}

// -------------------------------------------------- primitive accessors
// Triangle and 2D segment records behind one interface for the templates.
struct TriPrim {
    float3 pa, pb, pc;
    uint32_t index;
    FCPWGB_D static TriPrim load(const unsigned char *prims, uint32_t k) {
        const unsigned char *p = prims + (size_t)k * 40;
        float2 a = ldg2(p), b = ldg2(p + 8), c = ldg2(p + 16), d = ldg2(p + 24), e = ldg2(p + 32);
        TriPrim t;
        t.pa = make_float3(a.x, a.y, b.x);
        t.pb = make_float3(b.y, c.x, c.y);
        t.pc = make_float3(d.x, d.y, e.x);
        t.index = __float_as_uint(e.y);
        return t;
    }
    FCPWGB_HD float closestPoint(float3 x, float3 &p, float2 &uv) const {
        return closestPointTriangle(pa, pb, pc, x, p, uv);
    }
    FCPWGB_HD float3 normal() const { return normalize3(cross3(pb - pa, pc - pa)); }
    FCPWGB_HD float surfaceArea() const { return 0.5f * len3(cross3(pb - pa, pc - pa)); }
    FCPWGB_D bool intersect(const DevRay &r, bool occl, DevInteraction &i) const {
        return intersectTriangle(pa, pb, pc, r, occl, i);
    }
    // geometry.slang:410-424
    FCPWGB_HD float samplePoint(float2 rn, float2 &uv, float3 &p, float3 &n) const {
        n = cross3(pb - pa, pc - pa);
        float area = len3(n);
        float u1 = sqrtf(rn.x), u2 = rn.y;
        float u = 1.0f - u1, v = u2 * u1, w = 1.0f - u - v;
        uv = make_float2(u, v);
        p = pa * u + pb * v + pc * w;
        n = n / area;
        return 2.0f / area;
    }
};

struct SegPrim {
    float3 pa, pb;
    uint32_t index;
    FCPWGB_D static SegPrim load(const unsigned char *prims, uint32_t k) {
        // 24 B records start at 24k: 8 B aligned, so only 8 B vector loads
        const unsigned char *p = prims + (size_t)k * 24;
        float2 x = ldg2(p), y = ldg2(p + 8), z = ldg2(p + 16);
        SegPrim s;
        s.pa = make_float3(x.x, x.y, 0.0f);
        s.pb = make_float3(y.x, y.y, 0.0f);
        s.index = __float_as_uint(z.x);
        return s;
    }
    FCPWGB_HD float closestPoint(float3 x, float3 &p, float2 &uv) const {
        float t;
        float d = closestPointSegment(pa, pb, x, p, t);
        uv = make_float2(t, 0.0f);
        return d;
    }
    FCPWGB_HD float3 normal() const {
        float3 s = pb - pa;
        return normalize3(make_float3(s.y, -s.x, 0.0f));
    }
    FCPWGB_HD float surfaceArea() const { return len3(pb - pa); }
    FCPWGB_D bool intersect(const DevRay &r, bool occl, DevInteraction &i) const {
        return intersectSegment(pa, pb, r, occl, i);
    }
    // geometry.slang:183-193
    FCPWGB_HD float samplePoint(float2 rn, float2 &uv, float3 &p, float3 &n) const {
        float3 s = pb - pa;
        float area = len3(s);
        float u = rn.x;
        uv = make_float2(u, 0.0f);
        p = pa + s * u;
        n = make_float3(s.y, -s.x, 0.0f) / area;
        return 1.0f / area;
    }
};

}  // namespace fcpwgb
