// The reference CPU code's float arithmetic, rounding for rounding: every
// operation explicitly rounded to nearest (no fused multiply-adds), dot
// products and squared norms reduced as a0 + (a1 + a2) (the order of the
// unrolled fixed-size reductions the reference is compiled with). Ray-primitive
// tests written with these return the reference's hit distances, points,
// normals and uvs bit for bit, so hit indices differ from the reference only
// where the visiting order differs on an exact tie or a grazing hit.
//
// Included by device_common.cuh after its records (DevRay, DevInteraction).
#pragma once

namespace fcpwgb {

FCPWGB_D float3 xsub(float3 a, float3 b) {
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
FCPWGB_D float3 xadd(float3 a, float3 b) {
    return make_float3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
FCPWGB_D float3 xmul(float3 a, float s) { return make_float3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
FCPWGB_D float3 xdiv(float3 a, float s) { return make_float3(__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)); }
FCPWGB_D float xdot(int dim, float3 a, float3 b) {
    return dim == 3 ? __fadd_rn(__fmul_rn(a.x, b.x), __fadd_rn(__fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)))
                    : __fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
FCPWGB_D float3 xcross(float3 a, float3 b) {
    return make_float3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
                       __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
                       __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
// Vector::normalized(): divided by the square root of the squared norm when that is positive
FCPWGB_D float3 xnormalized(int dim, float3 a) {
    float z = xdot(dim, a, a);
    return z > 0.0f ? xdiv(a, __fsqrt_rn(z)) : a;
}

// Triangle::intersect (Moller-Trumbore), triangles.inl:222-260 (the GPU shader,
// geometry.slang:202-249, has the same operations); hits with 0 <= t <= tMax
FCPWGB_D bool xIntersectTriangle(float3 pa, float3 pb, float3 pc, const DevRay &r, bool occl, DevInteraction &i) {
    float3 v1 = xsub(pb, pa), v2 = xsub(pc, pa);
    float3 q0 = xcross(r.d, v2);
    float det = xdot(3, v1, q0);
    if (fabsf(det) <= kFltEps) return false;
    float invDet = __fdiv_rn(1.0f, det);
    float3 s = xsub(r.o, pa);
    float v = __fmul_rn(xdot(3, s, q0), invDet);
    if (v < 0.0f || v > 1.0f) return false;
    float3 q = xcross(s, v1);
    float w = __fmul_rn(xdot(3, r.d, q), invDet);
    if (w < 0.0f || __fadd_rn(v, w) > 1.0f) return false;
    float t = __fmul_rn(xdot(3, v2, q), invDet);
    if (!(t >= 0.0f && t <= r.tMax)) return false;
    if (occl) return true;
    i.d = t;
    i.p = xadd(xadd(pa, xmul(v1, v)), xmul(v2, w));
    i.n = xnormalized(3, xcross(v1, v2));
    i.uv = make_float2(__fsub_rn(__fsub_rn(1.0f, v), w), v);
    return true;
}

// LineSegment::intersect, line_segments.inl:140-175 (geometry.slang:37-77)
FCPWGB_D bool xIntersectSegment(float3 pa, float3 pb, const DevRay &r, bool occl, DevInteraction &i) {
    float3 u = xsub(pa, r.o), v = xsub(pb, pa);
    float dv = __fsub_rn(__fmul_rn(r.d.x, v.y), __fmul_rn(r.d.y, v.x));
    if (fabsf(dv) <= kFltEps) return false;
    float ud = __fsub_rn(__fmul_rn(u.x, r.d.y), __fmul_rn(u.y, r.d.x));
    float s = __fdiv_rn(ud, dv);
    if (!(s >= 0.0f && s <= 1.0f)) return false;
    float uv = __fsub_rn(__fmul_rn(u.x, v.y), __fmul_rn(u.y, v.x));
    float t = __fdiv_rn(uv, dv);
    if (!(t >= 0.0f && t <= r.tMax)) return false;
    if (occl) return true;
    i.d = t;
    i.p = xadd(pa, xmul(v, s));
    i.p.z = 0.0f;
    i.n = xnormalized(2, make_float3(v.y, -v.x, 0.0f));
    i.uv = make_float2(s, 0.0f);
    return true;
}

}  // namespace fcpwgb
