// Small fixed-size float vectors and boxes for the host BVH producer.
//
// The reference CPU code does this arithmetic through Eigen fixed-size
// expressions. Reductions over D coefficients (dot, squaredNorm, prod, sum)
// are evaluated by halving: a0 + (a1 + a2) for D = 3, which is the order of
// Eigen's unrolled fixed-size reduction. Element-wise min/max pick the second
// operand only when it compares strictly smaller/larger. Box padding is
// FLT_EPSILON as in include/fcpw/core/bounding_volumes.h:34-55.
#pragma once

#include <cfloat>
#include <cmath>

namespace fcpwgb {

template<int D> struct Vec {
    float c[D];
    float &operator[](int i) { return c[i]; }
    const float &operator[](int i) const { return c[i]; }
    static Vec constant(float v) { Vec r; for (int i = 0; i < D; i++) r.c[i] = v; return r; }
    static Vec zero() { return constant(0.0f); }
};

template<int D> inline Vec<D> operator+(const Vec<D> &a, const Vec<D> &b) { Vec<D> r; for (int i = 0; i < D; i++) r.c[i] = a.c[i] + b.c[i]; return r; }
template<int D> inline Vec<D> operator-(const Vec<D> &a, const Vec<D> &b) { Vec<D> r; for (int i = 0; i < D; i++) r.c[i] = a.c[i] - b.c[i]; return r; }
template<int D> inline Vec<D> operator*(const Vec<D> &a, float s) { Vec<D> r; for (int i = 0; i < D; i++) r.c[i] = a.c[i] * s; return r; }
template<int D> inline Vec<D> operator/(const Vec<D> &a, float s) { Vec<D> r; for (int i = 0; i < D; i++) r.c[i] = a.c[i] / s; return r; }
template<int D> inline Vec<D> &operator+=(Vec<D> &a, const Vec<D> &b) { for (int i = 0; i < D; i++) a.c[i] += b.c[i]; return a; }

inline float minf(float x, float y) { return y < x ? y : x; }
inline float maxf(float x, float y) { return x < y ? y : x; }

template<int D> inline Vec<D> cwiseMin(const Vec<D> &a, const Vec<D> &b) { Vec<D> r; for (int i = 0; i < D; i++) r.c[i] = minf(a.c[i], b.c[i]); return r; }
template<int D> inline Vec<D> cwiseMax(const Vec<D> &a, const Vec<D> &b) { Vec<D> r; for (int i = 0; i < D; i++) r.c[i] = maxf(a.c[i], b.c[i]); return r; }

// halving reductions
inline float redSum(const Vec<2> &a) { return a.c[0] + a.c[1]; }
inline float redSum(const Vec<3> &a) { return a.c[0] + (a.c[1] + a.c[2]); }
inline float redProd(const Vec<2> &a) { return a.c[0] * a.c[1]; }
inline float redProd(const Vec<3> &a) { return a.c[0] * (a.c[1] * a.c[2]); }
inline float dot(const Vec<2> &a, const Vec<2> &b) { return a.c[0] * b.c[0] + a.c[1] * b.c[1]; }
inline float dot(const Vec<3> &a, const Vec<3> &b) { return a.c[0] * b.c[0] + (a.c[1] * b.c[1] + a.c[2] * b.c[2]); }
template<int D> inline float squaredNorm(const Vec<D> &a) { return dot(a, a); }
template<int D> inline float norm(const Vec<D> &a) { return std::sqrt(squaredNorm(a)); }
template<int D> inline Vec<D> normalized(const Vec<D> &a) {
    float z = squaredNorm(a);
    return z > 0.0f ? a / std::sqrt(z) : a;
}
inline Vec<3> cross(const Vec<3> &a, const Vec<3> &b) {
    Vec<3> r;
    r.c[0] = a.c[1] * b.c[2] - a.c[2] * b.c[1];
    r.c[1] = a.c[2] * b.c[0] - a.c[0] * b.c[2];
    r.c[2] = a.c[0] * b.c[1] - a.c[1] * b.c[0];
    return r;
}

template<int D> struct Box {
    Vec<D> pMin = Vec<D>::constant(FLT_MAX);
    Vec<D> pMax = Vec<D>::constant(-FLT_MAX);

    static Box fromPoint(const Vec<D> &p) {
        Box b;
        Vec<D> e = Vec<D>::constant(FLT_EPSILON);
        b.pMin = p - e;
        b.pMax = p + e;
        return b;
    }
    void expand(const Vec<D> &p) {
        Vec<D> e = Vec<D>::constant(FLT_EPSILON);
        pMin = cwiseMin(pMin, p - e);
        pMax = cwiseMax(pMax, p + e);
    }
    void expand(const Box &b) {
        pMin = cwiseMin(pMin, b.pMin);
        pMax = cwiseMax(pMax, b.pMax);
    }
    Vec<D> extent() const { return pMax - pMin; }
    Vec<D> centroid() const { return (pMin + pMax) * 0.5f; }
    bool isValid() const { for (int i = 0; i < D; i++) if (!(pMax.c[i] >= pMin.c[i])) return false; return true; }
    int maxDimension() const {
        Vec<D> e = pMax - pMin;
        int index = 0;
        float best = e.c[0];
        for (int i = 1; i < D; i++) if (e.c[i] > best) { best = e.c[i]; index = i; }
        return index;
    }
    float surfaceArea() const {
        Vec<D> e = cwiseMax(extent(), Vec<D>::constant(1e-5f));
        float p = redProd(e);
        Vec<D> q;
        for (int i = 0; i < D; i++) q.c[i] = p / e.c[i];
        return 2.0f * redSum(q);
    }
    float volume() const { return redProd(extent()); }
    Box intersect(const Box &b) const {
        Box r;
        r.pMin = cwiseMax(pMin, b.pMin);
        r.pMax = cwiseMin(pMax, b.pMax);
        return r;
    }
};

}  // namespace fcpwgb
