// Silhouette primitives and the normal-cone overlap test used by the closest
// silhouette point query (geometry.slang:490-708, bounding-volumes.slang:118-232).
#pragma once

#include "device_common.cuh"

namespace fcpwgb {

FCPWGB_HD bool inRangeF(float v, float lo, float hi) { return v >= lo && v <= hi; }

// Frisvad-style branchless basis (Duff et al. 2017), bounding-volumes.slang:123-132
FCPWGB_HD void orthonormalBasis(float3 n, float3 &b1, float3 &b2) {
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    b1 = make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    b2 = make_float3(b, sign + n.y * n.y * a, -n.y);
}

FCPWGB_HD float projectToPlane3(float3 n, float3 e) {
    float3 b1, b2;
    orthonormalBasis(n, b1, b2);
    float r1 = dot3(e, make_float3(fabsf(b1.x), fabsf(b1.y), fabsf(b1.z)));
    float r2 = dot3(e, make_float3(fabsf(b2.x), fabsf(b2.y), fabsf(b2.z)));
    return sqrtf(r1 * r1 + r2 * r2);
}
// 2D case of the projection (bounding_volumes.h projectToPlane<2>)
FCPWGB_HD float projectToPlane2(float3 n, float3 e) {
    float r = e.x * fabsf(-n.y) + e.y * fabsf(n.x);
    return fabsf(r);
}

// cone vs view-cone overlap, bounding-volumes.slang:175-232
template<int DIM>
FCPWGB_HD bool coneOverlap(float3 axis, float halfAngle, float radius, float3 o, float3 bMin, float3 bMax,
                           float distToBox) {
    if (halfAngle >= kPi2F || distToBox < kFltEps) return true;
    float3 c = (bMin + bMax) * 0.5f;
    float3 viewConeAxis = c - o;
    float l = len3(viewConeAxis);
    viewConeAxis = viewConeAxis / l;
    float dAxisAngle = acosf(fmaxf(-1.0f, fminf(1.0f, dot3(axis, viewConeAxis))));
    if (inRangeF(kPi2F, dAxisAngle - halfAngle, dAxisAngle + halfAngle)) return true;
    if (l > radius) {
        float viewConeHalfAngle = asinf(radius / l);
        float halfAngleSum = halfAngle + viewConeHalfAngle;
        return halfAngleSum >= kPi2F ? true
                                     : inRangeF(kPi2F, dAxisAngle - halfAngleSum, dAxisAngle + halfAngleSum);
    }
    float3 e = bMax - c;
    float d = dot3(e, make_float3(fabsf(viewConeAxis.x), fabsf(viewConeAxis.y), fabsf(viewConeAxis.z)));
    float s = l - d;
    if (s <= 0.0f) return true;
    d = DIM == 3 ? projectToPlane3(viewConeAxis, e) : projectToPlane2(viewConeAxis, e);
    float viewConeHalfAngle = atan2f(d, s);
    float halfAngleSum = halfAngle + viewConeHalfAngle;
    return halfAngleSum >= kPi2F ? true
                                 : inRangeF(kPi2F, dAxisAngle - halfAngleSum, dAxisAngle + halfAngleSum);
}

// The same decision as coneOverlap without its inverse trigonometric functions
// wherever a margin makes the answer certain. With x = |axis . v| (v the unit
// view-cone axis), h the cone's half angle and phi the view cone's half angle,
// coneOverlap's test |acos(x') - pi/2| <= h + phi (x' the signed dot product)
// is |asin(x')| <= H, H = h + phi, i.e. x <= sin(H) while H < pi/2, and
// H >= pi/2 means sin(phi) >= cos(h). In sine space: sin(phi) = radius / l
// (l > radius) or d / sqrt(d^2 + s^2) (the box's projected half extent d at
// distance s), sin(H) = sin h cos phi + cos h sin phi, and sin h, cos h by
// the fast intrinsics (absolute error below 1e-6 on [0, pi/2)). Every
// comparison is decided only when it clears kConeMargin = 1e-5, which exceeds
// the rounding of both evaluations by more than ten times (the dot product,
// the intrinsics, and coneOverlap's acos / asin / atan2 and angle sums, each
// within a few 2^-24 in sine space); otherwise coneOverlap itself decides. So
// the outcome is coneOverlap's, with the transcendental functions evaluated
// only for boxes within 1e-5 of the cone's boundary.
constexpr float kConeMargin = 1e-5f;
template<int DIM>
FCPWGB_D bool coneOverlapFast(float3 axis, float halfAngle, float radius, float3 o, float3 bMin, float3 bMax,
                              float distToBox) {
    if (halfAngle >= kPi2F || distToBox < kFltEps) return true;
    const float3 c = (bMin + bMax) * 0.5f;
    float3 v = c - o;
    const float l = len3(v);
    v = v / l;
    const float x = fabsf(fmaxf(-1.0f, fminf(1.0f, dot3(axis, v))));
    const float sh = __sinf(halfAngle), ch = __cosf(halfAngle);
    if (x <= sh - kConeMargin) return true;  // the first test: |acos - pi/2| <= h
    float sp, cp;
    if (l > radius) {
        sp = radius / l;
        cp = sqrtf(fmaxf(0.0f, 1.0f - sp * sp));
    } else {
        const float3 e = bMax - c;
        const float d = dot3(e, make_float3(fabsf(v.x), fabsf(v.y), fabsf(v.z)));
        const float s = l - d;
        if (s <= 0.0f) return true;
        const float dp = DIM == 3 ? projectToPlane3(v, e) : projectToPlane2(v, e);
        const float nrm = sqrtf(dp * dp + s * s);
        sp = dp / nrm;
        cp = s / nrm;
    }
    if (sp >= ch + kConeMargin) return true;  // h + phi >= pi/2
    if (sp > ch - kConeMargin) return coneOverlap<DIM>(axis, halfAngle, radius, o, bMin, bMax, distToBox);
    const float sH = sh * cp + ch * sp;
    if (x <= sH - kConeMargin) return true;
    if (x >= sH + kConeMargin) return false;
    return coneOverlap<DIM>(axis, halfAngle, radius, o, bMin, bMax, distToBox);
}

// geometry.slang:490-522
FCPWGB_HD bool isSilhouetteVertex(float3 n0, float3 n1, float3 viewDir, float d, bool flip, float precision) {
    float sign = flip ? 1.0f : -1.0f;
    if (d <= precision) {
        float det = n0.x * n1.y - n1.x * n0.y;
        return sign * det > precision;
    }
    float3 vd = viewDir / d;
    float dot0 = dot3(vd, n0), dot1 = dot3(vd, n1);
    if (fabsf(dot0) <= precision) return sign * dot1 > precision;
    if (fabsf(dot1) <= precision) return sign * dot0 > precision;
    return dot0 * dot1 < 0.0f;
}

// geometry.slang:599-633
FCPWGB_HD bool isSilhouetteEdge(float3 pa, float3 pb, float3 n0, float3 n1, float3 viewDir, float d, bool flip,
                                float precision) {
    float sign = flip ? 1.0f : -1.0f;
    if (d <= precision) {
        float3 edgeDir = normalize3(pb - pa);
        float signedDihedralAngle = atan2f(dot3(edgeDir, cross3(n0, n1)), dot3(n0, n1));
        return sign * signedDihedralAngle > precision;
    }
    float3 vd = viewDir / d;
    float dot0 = dot3(vd, n0), dot1 = dot3(vd, n1);
    if (fabsf(dot0) <= precision) return sign * dot1 > precision;
    if (fabsf(dot1) <= precision) return sign * dot0 > precision;
    return dot0 * dot1 < 0.0f;
}

struct EdgeSil {
    float3 pa, pb, n0, n1;
    uint32_t index, hasOne;
    FCPWGB_D static EdgeSil load(const unsigned char *sils, uint32_t k) {
        const unsigned char *p = sils + (size_t)k * 56;
        float2 a = ldg2(p), b = ldg2(p + 8), c = ldg2(p + 16), d = ldg2(p + 24), e = ldg2(p + 32),
               f = ldg2(p + 40), g = ldg2(p + 48);
        EdgeSil s;
        s.pa = make_float3(a.x, a.y, b.x);
        s.pb = make_float3(b.y, c.x, c.y);
        s.n0 = make_float3(d.x, d.y, e.x);
        s.n1 = make_float3(e.y, f.x, f.y);
        s.index = __float_as_uint(g.x);
        s.hasOne = __float_as_uint(g.y);
        return s;
    }
    // geometry.slang:668-701
    FCPWGB_HD bool closestSilhouettePoint(float3 c, float r2, bool flip, float sqMinR, float precision,
                                          DevInteraction &i) const {
        if (sqMinR >= r2) return false;
        float t;
        float d = closestPointSegment(pa, pb, c, i.p, t);
        i.uv.x = t;
        if (d * d > r2) return false;
        bool process = hasOne == 1;
        if (!process) process = isSilhouetteEdge(pa, pb, n0, n1, c - i.p, d, flip, precision);
        if (process && d * d <= r2) {
            i.uv.y = 0.0f;
            i.d = d;
            i.index = index;
            return true;
        }
        return false;
    }
};

struct VertexSil {
    float3 p, n0, n1;
    uint32_t index, hasOne;
    FCPWGB_D static VertexSil load(const unsigned char *sils, uint32_t k) {
        const unsigned char *q = sils + (size_t)k * 32;
        float4 a = ldg4(q), b = ldg4(q + 16);
        VertexSil s;
        s.p = make_float3(a.x, a.y, 0.0f);
        s.n0 = make_float3(a.z, a.w, 0.0f);
        s.n1 = make_float3(b.x, b.y, 0.0f);
        s.index = __float_as_uint(b.z);
        s.hasOne = __float_as_uint(b.w);
        return s;
    }
    // geometry.slang:556-590
    FCPWGB_HD bool closestSilhouettePoint(float3 c, float r2, bool flip, float sqMinR, float precision,
                                          DevInteraction &i) const {
        if (sqMinR >= r2) return false;
        float3 viewDir = c - p;
        float d = len3(viewDir);
        if (d * d > r2) return false;
        bool process = hasOne == 1;
        if (!process) process = isSilhouetteVertex(n0, n1, viewDir, d, flip, precision);
        if (process && d * d <= r2) {
            i.p = p;
            i.uv = make_float2(0.0f, 0.0f);
            i.d = d;
            i.index = index;
            return true;
        }
        return false;
    }
};

}  // namespace fcpwgb
