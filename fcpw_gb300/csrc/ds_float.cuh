// Double-single ("pair of floats") arithmetic for the precise closest-point
// refinement. A value is hi + lo with |lo| <= ulp(hi)/2; sums and products
// carry about 44-48 significant bits, on the FP32 pipes, which run many
// times faster than FP64 on this part.
//
// Methods (published, restated here from their mathematics):
//  - TwoSum: Knuth, The Art of Computer Programming vol. 2, 4.2.2 (exact
//    sum of two floats as hi + lo, no ordering needed);
//  - FastTwoSum and the pair sum, product, quotient and square root:
//    T. J. Dekker, "A floating-point technique for extending the available
//    precision", Numerische Mathematik 18 (1971); the quotient takes one
//    correction step q2 = (a - q1 b) / b, the square root one Newton step
//    e = (a - s^2) / 2s on s = sqrt(a.hi);
//  - TwoProd by a fused multiply-add (the exact error of a rounded
//    product is fma(a, b, -ab)).
// Every step uses the _rn intrinsics so the compiler neither contracts nor
// reorders the error terms; division and square root of the leading parts
// are CUDA's IEEE round-to-nearest operations.
#pragma once

#include "device_common.cuh"

namespace fcpwgb {

struct DS {
    float hi, lo;
};

FCPWGB_D DS dsOf(float a) { return DS{a, 0.0f}; }

// exact a + b
FCPWGB_D DS twoSum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return DS{s, e};
}

// exact a + b when |a| >= |b| (or a == 0)
FCPWGB_D DS fastTwoSum(float a, float b) {
    float s = __fadd_rn(a, b);
    return DS{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// exact a * b (barring underflow)
FCPWGB_D DS twoProd(float a, float b) {
    float p = __fmul_rn(a, b);
    return DS{p, __fmaf_rn(a, b, -p)};
}

FCPWGB_D DS dsNeg(DS a) { return DS{-a.hi, -a.lo}; }

// pair sum with both low parts added separately (accurate also when the
// leading parts cancel)
FCPWGB_D DS dsAdd(DS a, DS b) {
    DS s = twoSum(a.hi, b.hi);
    DS t = twoSum(a.lo, b.lo);
    s = fastTwoSum(s.hi, __fadd_rn(s.lo, t.hi));
    return fastTwoSum(s.hi, __fadd_rn(s.lo, t.lo));
}
FCPWGB_D DS dsSub(DS a, DS b) { return dsAdd(a, dsNeg(b)); }

FCPWGB_D DS dsMul(DS a, DS b) {
    DS p = twoProd(a.hi, b.hi);
    float lo = __fmaf_rn(a.hi, b.lo, p.lo);
    lo = __fmaf_rn(a.lo, b.hi, lo);
    return fastTwoSum(p.hi, lo);
}

FCPWGB_D DS dsMulF(DS a, float b) {
    DS p = twoProd(a.hi, b);
    return fastTwoSum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

FCPWGB_D DS dsDiv(DS a, DS b) {
    float q1 = __fdiv_rn(a.hi, b.hi);
    DS r = dsSub(a, dsMulF(b, q1));
    float q2 = __fdiv_rn(r.hi, b.hi);
    return fastTwoSum(q1, q2);
}

FCPWGB_D DS dsSqrt(DS a) {
    if (a.hi <= 0.0f) return DS{0.0f, 0.0f};
    float s = __fsqrt_rn(a.hi);
    DS r = dsSub(a, twoProd(s, s));
    return fastTwoSum(s, __fdiv_rn(r.hi, __fmul_rn(2.0f, s)));
}

FCPWGB_D DS dsDot3(DS ax, DS ay, DS az, DS bx, DS by, DS bz) {
    return dsAdd(dsAdd(dsMul(ax, bx), dsMul(ay, by)), dsMul(az, bz));
}

// the pair nearest to an FP64 value
FCPWGB_D DS dsFromDouble(double d) {
    float hi = (float)d;
    return DS{hi, (float)(d - (double)hi)};
}

}  // namespace fcpwgb
