// Closest-point traversal of the wide / quantised trees (wide.h), plus the
// device re-quantisation after a refit. Templates only; instantiated per
// branching factor in k_wide_w{2,4,8}.cu.
#pragma once

#include <type_traits>

#include "ds_float.cuh"
#include "kernels.h"
#include "wide_common.cuh"

namespace fcpwgb {

// Bounds of the double-single refinement (refine below): conditioning limit
// (2^-46 x 2^10 = 2^-36 relative error at most, far below the 1e-6 that the
// precise mode promises) and the ranges of the offset scale, the edges and
// the normal within which squares and products of pairs stay normal floats.
constexpr float kDsCond = 1024.0f;
// relative margin by which a refined runner-up must beat the refined winner
// (above the refinement's rounding, far below the 1e-6 accuracy promised)
constexpr float kRefineTie = 0x1p-28f;
constexpr float kDsMinScale = 0x1p-28f, kDsMaxScale = 0x1p28f, kDsMinEdge = 0x1p-30f, kDsMinNormal = 0x1p-40f;

// 48 B triangle record of the wide kernels: (pa, index), (pb, 0), (pc, 0)
struct Tri48Prim {
    // precise mode refines in a second pass (kRefineClosest): inlined at the
    // end of the traversal, the triangle refinement made the traversal loop
    // spill
    static constexpr bool kRefinePass = true;
    float3 pa, pb, pc;
    uint32_t index;
    FCPWGB_D static Tri48Prim load(const unsigned char *prims, uint32_t k) {
        const unsigned char *p = prims + (size_t)k * 48;
        float4 a = ldg4(p), b = ldg4(p + 16), c = ldg4(p + 32);
        Tri48Prim t;
        t.pa = make_float3(a.x, a.y, a.z);
        t.pb = make_float3(b.x, b.y, b.z);
        t.pc = make_float3(c.x, c.y, c.z);
        t.index = __float_as_uint(a.w);
        return t;
    }
    FCPWGB_D float closestPoint(float3 x, float3 &p, float2 &uv) const {
        return closestPointTriangle(pa, pb, pc, x, p, uv);
    }
    FCPWGB_D float3 normal() const { return normalize3(cross3(pb - pa, pc - pa)); }
    FCPWGB_D bool intersect(const DevRay &r, bool occl, DevInteraction &i) const {
        return intersectTriangle(pa, pb, pc, r, occl, i);
    }
    // FP64 distance and closest point, vertices taken relative to the query
    // (not inlined: its FP64 registers stay out of the traversal loop)
    __device__ __noinline__ double refine64(float3 x, float3 &pOut) const {
        double ax = (double)pa.x - x.x, ay = (double)pa.y - x.y, az = (double)pa.z - x.z;
        double bx = (double)pb.x - x.x, by = (double)pb.y - x.y, bz = (double)pb.z - x.z;
        double cx = (double)pc.x - x.x, cy = (double)pc.y - x.y, cz = (double)pc.z - x.z;
        double abx = bx - ax, aby = by - ay, abz = bz - az, acx = cx - ax, acy = cy - ay, acz = cz - az;
        double px, py, pz;
        double d1 = -(abx * ax + aby * ay + abz * az), d2 = -(acx * ax + acy * ay + acz * az);
        double d3 = -(abx * bx + aby * by + abz * bz), d4 = -(acx * bx + acy * by + acz * bz);
        double d5 = -(abx * cx + aby * cy + abz * cz), d6 = -(acx * cx + acy * cy + acz * cz);
        double vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
        if (d1 <= 0 && d2 <= 0) { px = ax; py = ay; pz = az; }
        else if (d3 >= 0 && d4 <= d3) { px = bx; py = by; pz = bz; }
        else if (d6 >= 0 && d5 <= d6) { px = cx; py = cy; pz = cz; }
        else if (vc <= 0 && d1 >= 0 && d3 <= 0) {
            double v = d1 / (d1 - d3);
            px = ax + abx * v; py = ay + aby * v; pz = az + abz * v;
        } else if (vb <= 0 && d2 >= 0 && d6 <= 0) {
            double w = d2 / (d2 - d6);
            px = ax + acx * w; py = ay + acy * w; pz = az + acz * w;
        } else if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
            double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            px = bx + (cx - bx) * w; py = by + (cy - by) * w; pz = bz + (cz - bz) * w;
        } else {
            // face region: project the query (the origin) onto the plane
            double nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
            double nn = nx * nx + ny * ny + nz * nz;
            double t = (ax * nx + ay * ny + az * nz) / nn;
            px = nx * t; py = ny * t; pz = nz * t;
        }
        pOut = make_float3((float)(x.x + px), (float)(x.y + py), (float)(x.z + pz));
        return sqrt(px * px + py * py + pz * pz);
    }
    // The same distance and closest point in double-single arithmetic
    // (ds_float.cuh), which runs on the FP32 pipes. The vertex offsets
    // from the query and the edges are exact pairs (TwoSum), so the error
    // grows only with the conditioning of the projection,
    // cond = s |ab| |ac| / (|n| d), s the largest vertex offset, n the
    // face normal and d the FP32 distance found by the traversal: about
    // 2^-46 cond relative. Where the FP32 estimate of cond is above
    // kDsCond, or s, an edge or |n| lies outside the range where pair
    // products stay normal floats, refine64 computes it in FP64 instead.
    FCPWGB_D DS refine(float3 x, float dApprox, float3 &pOut) const {
        const float3 eab = pb - pa, eac = pc - pa, ebc = pc - pb;
        const float s = fmaxf(fmaxf(fmaxf(fabsf(pa.x - x.x), fabsf(pa.y - x.y)), fmaxf(fabsf(pa.z - x.z),
                                    fabsf(pb.x - x.x))),
                              fmaxf(fmaxf(fabsf(pb.y - x.y), fabsf(pb.z - x.z)),
                                    fmaxf(fmaxf(fabsf(pc.x - x.x), fabsf(pc.y - x.y)), fabsf(pc.z - x.z))));
        const float lab = len3(eab), lac = len3(eac), ln = len3(cross3(eab, eac));
        const bool ok = s >= kDsMinScale && s <= kDsMaxScale && fminf(fminf(lab, lac), len3(ebc)) >= kDsMinEdge &&
                        ln >= kDsMinNormal && s * lab * lac <= kDsCond * ln * dApprox;
        if (!ok) return dsFromDouble(refine64(x, pOut));
        const DS ax = twoSum(pa.x, -x.x), ay = twoSum(pa.y, -x.y), az = twoSum(pa.z, -x.z);
        const DS bx = twoSum(pb.x, -x.x), by = twoSum(pb.y, -x.y), bz = twoSum(pb.z, -x.z);
        const DS cx = twoSum(pc.x, -x.x), cy = twoSum(pc.y, -x.y), cz = twoSum(pc.z, -x.z);
        const DS abx = twoSum(pb.x, -pa.x), aby = twoSum(pb.y, -pa.y), abz = twoSum(pb.z, -pa.z);
        const DS acx = twoSum(pc.x, -pa.x), acy = twoSum(pc.y, -pa.y), acz = twoSum(pc.z, -pa.z);
        const DS d1 = dsNeg(dsDot3(abx, aby, abz, ax, ay, az)), d2 = dsNeg(dsDot3(acx, acy, acz, ax, ay, az));
        const DS d3 = dsNeg(dsDot3(abx, aby, abz, bx, by, bz)), d4 = dsNeg(dsDot3(acx, acy, acz, bx, by, bz));
        const DS d5 = dsNeg(dsDot3(abx, aby, abz, cx, cy, cz)), d6 = dsNeg(dsDot3(acx, acy, acz, cx, cy, cz));
        DS px, py, pz;
        if (d1.hi <= 0.0f && d2.hi <= 0.0f) {
            px = ax; py = ay; pz = az;
        } else if (d3.hi >= 0.0f && dsSub(d4, d3).hi <= 0.0f) {
            px = bx; py = by; pz = bz;
        } else if (d6.hi >= 0.0f && dsSub(d5, d6).hi <= 0.0f) {
            px = cx; py = cy; pz = cz;
        } else {
            const DS vc = dsSub(dsMul(d1, d4), dsMul(d3, d2));
            const DS vb = dsSub(dsMul(d5, d2), dsMul(d1, d6));
            const DS va = dsSub(dsMul(d3, d6), dsMul(d5, d4));
            const DS e43 = dsSub(d4, d3), e56 = dsSub(d5, d6);
            if (vc.hi <= 0.0f && d1.hi >= 0.0f && d3.hi <= 0.0f) {
                const DS v = dsDiv(d1, dsSub(d1, d3));
                px = dsAdd(ax, dsMul(abx, v)); py = dsAdd(ay, dsMul(aby, v)); pz = dsAdd(az, dsMul(abz, v));
            } else if (vb.hi <= 0.0f && d2.hi >= 0.0f && d6.hi <= 0.0f) {
                const DS w = dsDiv(d2, dsSub(d2, d6));
                px = dsAdd(ax, dsMul(acx, w)); py = dsAdd(ay, dsMul(acy, w)); pz = dsAdd(az, dsMul(acz, w));
            } else if (va.hi <= 0.0f && e43.hi >= 0.0f && e56.hi >= 0.0f) {
                const DS w = dsDiv(e43, dsAdd(e43, e56));
                px = dsAdd(bx, dsMul(twoSum(pc.x, -pb.x), w));
                py = dsAdd(by, dsMul(twoSum(pc.y, -pb.y), w));
                pz = dsAdd(bz, dsMul(twoSum(pc.z, -pb.z), w));
            } else {
                // face region: project the query (the origin) onto the plane
                const DS nx = dsSub(dsMul(aby, acz), dsMul(abz, acy));
                const DS ny = dsSub(dsMul(abz, acx), dsMul(abx, acz));
                const DS nz = dsSub(dsMul(abx, acy), dsMul(aby, acx));
                const DS t = dsDiv(dsDot3(ax, ay, az, nx, ny, nz), dsDot3(nx, ny, nz, nx, ny, nz));
                px = dsMul(nx, t); py = dsMul(ny, t); pz = dsMul(nz, t);
            }
        }
        pOut = make_float3(dsAdd(dsOf(x.x), px).hi, dsAdd(dsOf(x.y), py).hi, dsAdd(dsOf(x.z), pz).hi);
        return dsSqrt(dsDot3(px, py, pz, px, py, pz));
    }
};

// 2D segments keep the 24 B record (SegPrim) and gain the refinement
struct Seg24Prim : SegPrim {
    // precise mode refines at the end of the traversal: the segment
    // refinement is small enough (no spills), and a second pass over all
    // records would cost more than it does
    static constexpr bool kRefinePass = false;
    FCPWGB_D static Seg24Prim load(const unsigned char *prims, uint32_t k) {
        Seg24Prim s;
        SegPrim b = SegPrim::load(prims, k);
        s.pa = b.pa; s.pb = b.pb; s.index = b.index;
        return s;
    }
    __device__ __noinline__ double refine64(float3 x, float3 &pOut) const {
        double ax = (double)pa.x - x.x, ay = (double)pa.y - x.y;
        double ux = (double)pb.x - pa.x, uy = (double)pb.y - pa.y;
        double c1 = -(ux * ax + uy * ay), c2 = ux * ux + uy * uy, px, py;
        if (c1 <= 0) { px = ax; py = ay; }
        else if (c2 <= c1) { px = ax + ux; py = ay + uy; }
        else { double t = c1 / c2; px = ax + ux * t; py = ay + uy * t; }
        pOut = make_float3((float)(x.x + px), (float)(x.y + py), 0.0f);
        return sqrt(px * px + py * py);
    }
    // double-single counterpart (see Tri48Prim::refine); a segment's
    // projection has cond = s / d (not inlined: it runs inside the traversal
    // kernels, whose loops keep their registers)
    __device__ __noinline__ DS refine(float3 x, float dApprox, float3 &pOut) const {
        const float s = fmaxf(fmaxf(fabsf(pa.x - x.x), fabsf(pa.y - x.y)), fmaxf(fabsf(pb.x - x.x), fabsf(pb.y - x.y)));
        const bool ok = s >= kDsMinScale && s <= kDsMaxScale && len3(pb - pa) >= kDsMinEdge &&
                        s <= kDsCond * dApprox;
        if (!ok) return dsFromDouble(refine64(x, pOut));
        const DS ax = twoSum(pa.x, -x.x), ay = twoSum(pa.y, -x.y);
        const DS ux = twoSum(pb.x, -pa.x), uy = twoSum(pb.y, -pa.y);
        const DS c1 = dsNeg(dsAdd(dsMul(ux, ax), dsMul(uy, ay))), c2 = dsAdd(dsMul(ux, ux), dsMul(uy, uy));
        DS px, py;
        if (c1.hi <= 0.0f) {
            px = ax; py = ay;
        } else if (dsSub(c2, c1).hi <= 0.0f) {
            px = dsAdd(ax, ux); py = dsAdd(ay, uy);
        } else {
            const DS t = dsDiv(c1, c2);
            px = dsAdd(ax, dsMul(ux, t)); py = dsAdd(ay, dsMul(uy, t));
        }
        pOut = make_float3(dsAdd(dsOf(x.x), px).hi, dsAdd(dsOf(x.y), py).hi, 0.0f);
        return dsSqrt(dsAdd(dsMul(px, px), dsMul(py, py)));
    }
};

template<int W, int BITS> struct WideNodeRegs {
    using L = WideLayout<W, BITS>;
    static constexpr int kWords = L::kSize / 4;
    uint32_t w[kWords];

    FCPWGB_D void load(const unsigned char *nodes, uint32_t idx) {
        const uint4 *p = reinterpret_cast<const uint4 *>(nodes + (size_t)idx * L::kSize);
#pragma unroll
        for (int i = 0; i < kWords / 4; i++) {
            uint4 v = __ldg(p + i);
            w[4 * i] = v.x; w[4 * i + 1] = v.y; w[4 * i + 2] = v.z; w[4 * i + 3] = v.w;
        }
    }
    FCPWGB_D uint32_t byteAt(int off) const { return (w[off >> 2] >> (8 * (off & 3))) & 0xffu; }
    FCPWGB_D uint32_t halfAt(int off) const { return (w[off >> 2] >> (8 * (off & 3))) & 0xffffu; }
    FCPWGB_D uint32_t ref(int c) const { return w[(L::kRefs >> 2) + c]; }
    FCPWGB_D uint32_t cnt(int c) const { return byteAt(L::kCnt + c); }
    // cnt of a runtime slot (< W) by shifts, without indexing the registers:
    // the count bytes start on a word, one word for W <= 4, two for W = 8
    FCPWGB_D uint32_t cntAt(uint32_t slot) const {
        static_assert((L::kCnt & 3) == 0, "count bytes start on a word");
        if constexpr (W <= 4) {
            return (w[L::kCnt >> 2] >> (8u * slot)) & 0xffu;
        } else {
            const uint64_t b = (uint64_t)w[L::kCnt >> 2] | ((uint64_t)w[(L::kCnt >> 2) + 1] << 32);
            return (uint32_t)(b >> (8u * slot)) & 0xffu;
        }
    }
    FCPWGB_D float origin(int a) const { return __uint_as_float(w[a]); }
    FCPWGB_D float scale(int a) const { return exp2i((int)byteAt(12 + a) - 127); }
    // bound k = 0..2 lo(x,y,z), 3..5 hi(x,y,z) of child c
    FCPWGB_D float bound(int k, int c) const {
        if (BITS == 32) return __uint_as_float(w[(L::kBounds >> 2) + k * W + c]);
        int a = k % 3;
        return __fmaf_rn(qvalue(k, c), scale(a), origin(a));
    }
    // the quantised integer of bound k of child c as a float: one byte permute
    // places q (< 2^16) in the low mantissa bits of 2^23, then the bias is
    // subtracted (exact)
    FCPWGB_D float qvalue(int k, int c) const {
        const int off = BITS == 16 ? L::kBounds + 2 * (k * W + c) : L::kBounds + k * W + c;
        const uint32_t b = (uint32_t)(off & 3);
        const uint32_t sel = BITS == 16 ? (0x7400u | ((b + 1u) << 4) | b) : (0x7440u | b);
        return __uint_as_float(__byte_perm(w[off >> 2], 0x4b000000u, sel)) - 8388608.0f;
    }
};

// Squared min distances from query c to the W children of a node, and the
// squared max distance to child k, on the dequantised boxes
// fmaf(q, 2^e, origin) -- the exact values the quantiser checked to contain
// each child.
FCPWGB_D float fmax3(float a, float b, float c) {  // three-input max (sm_100+)
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
template<int W, int BITS>
FCPWGB_D void childD2Min(const WideNodeRegs<W, BITS> &node, float3 c, float (&d2Min)[W]) {
#pragma unroll
    for (int k = 0; k < W; k++) {
        // boxSphereD2Min with the per-axis max(lo - c, c - hi, 0) in one instruction
        float ax = fmax3(node.bound(0, k) - c.x, c.x - node.bound(3, k), 0.0f);
        float ay = fmax3(node.bound(1, k) - c.y, c.y - node.bound(4, k), 0.0f);
        float az = fmax3(node.bound(2, k) - c.z, c.z - node.bound(5, k), 0.0f);
        d2Min[k] = ax * ax + ay * ay + az * az;
    }
}
template<int W, int BITS>
FCPWGB_D float childD2Max(const WideNodeRegs<W, BITS> &node, float3 c, int k) {
    float lo, hi;
    boxSphereDist(make_float3(node.bound(0, k), node.bound(1, k), node.bound(2, k)),
                  make_float3(node.bound(3, k), node.bound(4, k), node.bound(5, k)), c, lo, hi);
    return hi;
}

constexpr uint32_t kLeafBit = 0x80000000u;

// the search radius of a query: empty (-1) when its centre is not finite,
// since the box distances drop NaN operands (max.f32) and would admit every
// box, or when the radius itself is NaN, which the first shrink to a child's
// far distance (fminf drops NaN) would turn finite; such a query gets the
// default record without walking the tree, as in the reference, whose root
// test d2Min <= r2 fails for a NaN radius
FCPWGB_D float queryRadius2(float3 c, float r2) {
    return isfinite(c.x) && isfinite(c.y) && isfinite(c.z) && r2 == r2 ? r2 : -1.0f;
}
FCPWGB_D uint32_t packLeaf(uint32_t off, uint32_t cnt) { return kLeafBit | (cnt << 27) | off; }

// a[slot] for a register array and a runtime slot < W: a binary tree of
// selects on the slot's bits (W - 1 selects) instead of W compare-and-selects
template<int W, class T> FCPWGB_D T selectBySlot(const T (&a)[W], uint32_t slot) {
    if constexpr (W == 2) {
        return (slot & 1u) ? a[1] : a[0];
    } else if constexpr (W == 4) {
        T lo = (slot & 1u) ? a[1] : a[0], hi = (slot & 1u) ? a[3] : a[2];
        return (slot & 2u) ? hi : lo;
    } else {
        T q0 = (slot & 1u) ? a[1] : a[0], q1 = (slot & 1u) ? a[3] : a[2];
        T q2 = (slot & 1u) ? a[5] : a[4], q3 = (slot & 1u) ? a[7] : a[6];
        T h0 = (slot & 2u) ? q1 : q0, h1 = (slot & 2u) ? q3 : q2;
        return (slot & 4u) ? h1 : h0;
    }
}

// the stack reference of every child slot: inner record index, or a packed leaf
template<int W, int BITS> FCPWGB_D void childRefs(const WideNodeRegs<W, BITS> &node, uint32_t (&packed)[W]) {
#pragma unroll
    for (int s = 0; s < W; s++) {
        uint32_t n = node.cnt(s);
        packed[s] = n == 0 ? node.ref(s) : packLeaf(node.ref(s), n);
    }
}

// Sorting networks over packed keys (non-negative float bits with the child
// slot in the low bits): integer min/max compare-exchanges. Optimal networks
// for 2, 4 (5 comparators) and 8 (19 comparators) inputs.
FCPWGB_D void cmpx(uint32_t &a, uint32_t &b) {
    uint32_t lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}
template<int W> FCPWGB_D void sortNetwork(uint32_t (&k)[W]);
template<> FCPWGB_D void sortNetwork<2>(uint32_t (&k)[2]) { cmpx(k[0], k[1]); }
template<> FCPWGB_D void sortNetwork<4>(uint32_t (&k)[4]) {
    cmpx(k[0], k[1]); cmpx(k[2], k[3]); cmpx(k[0], k[2]); cmpx(k[1], k[3]); cmpx(k[1], k[2]);
}
template<> FCPWGB_D void sortNetwork<8>(uint32_t (&k)[8]) {
    cmpx(k[0], k[2]); cmpx(k[1], k[3]); cmpx(k[4], k[6]); cmpx(k[5], k[7]);
    cmpx(k[0], k[4]); cmpx(k[1], k[5]); cmpx(k[2], k[6]); cmpx(k[3], k[7]);
    cmpx(k[0], k[1]); cmpx(k[2], k[3]); cmpx(k[4], k[5]); cmpx(k[6], k[7]);
    cmpx(k[2], k[4]); cmpx(k[3], k[5]);
    cmpx(k[1], k[4]); cmpx(k[3], k[6]);
    cmpx(k[1], k[2]); cmpx(k[3], k[4]); cmpx(k[5], k[6]);
}

// Per-thread traversal stack of kWideStack entries (node reference + the
// child's distance bound). With SHORT = 16 the first 16 entries live in
// shared memory, entry k of thread t at [k * 128 + t] so that a warp's
// accesses fall in distinct banks, and deeper entries go to local memory,
// which only deep traversals touch; with SHORT = 0 the whole stack is in
// local memory. A whole stack in local memory (1 KB per thread) does not fit
// the L1 of a fully occupied SM and its pushes and pops reach L2 and DRAM.
constexpr int kShortStack = 16;
constexpr int kWideBlock = 128;  // threads per block of the wide kernels
template<int SHORT> struct WideStack {
    uint32_t *sRef;  // shared, stride kWideBlock
    float *sD;
    uint32_t lRef[kWideStack - SHORT];
    float lD[kWideStack - SHORT];
    FCPWGB_D void push(int sp, uint32_t ref, float d) {
        if (sp < SHORT) {
            sRef[sp * kWideBlock] = ref;
            sD[sp * kWideBlock] = d;
        } else {
            lRef[sp - SHORT] = ref;
            lD[sp - SHORT] = d;
        }
    }
    FCPWGB_D float dist(int sp) const { return sp < SHORT ? sD[sp * kWideBlock] : lD[sp - SHORT]; }
    FCPWGB_D uint32_t ref(int sp) const { return sp < SHORT ? sRef[sp * kWideBlock] : lRef[sp - SHORT]; }
};

// Traversal statistics (expansions, tests, warp loads): compiled in only for
// the counting launches, so the timed kernels carry no counter registers.
template<bool ON> struct Count {
    FCPWGB_D void add(uint32_t) {}
    FCPWGB_D unsigned long long get() const { return 0; }
};
template<> struct Count<true> {
    uint32_t v = 0;
    FCPWGB_D void add(uint32_t x) { v += x; }
    FCPWGB_D unsigned long long get() const { return v; }
};

// Rounding band of a distance. The band, 8 units of 2^-24 times
// (|c|_inf + d), bounds the FP32 error of a point-primitive or point-box
// distance with coordinates of magnitude |c| + d. Boxes are visited while
// their distance is within the winner's distance plus the band (in every
// mode): a box holding a primitive at exactly the winner's distance can then
// not be pruned by rounding, which at query coordinates much larger than the
// box padding (FLT_EPSILON) would otherwise happen, and exact ties resolve
// by the rule of beatsWinner whatever the visiting order.
//
// Near ties of the precise mode. The FP32 traversal picks its winner with the
// reference's rounding, but a primitive whose FP32 distance lies within the
// band of the winner's may be the closer one in exact arithmetic. So the
// precise mode also keeps the best primitive within the band other than the
// winner (the runner-up) and refines both at the end (Tri48Prim::refine:
// double-single arithmetic, FP64 where ill-conditioned). Without it,
// near-tied segments of a polyline gave 7.5e-7 relative error on 1024 2D
// samples.
constexpr float kBandEps = 8.0f * 5.9604645e-8f;
FCPWGB_D float tieBand(float3 c, float d) { return kBandEps * (fmax3(fabsf(c.x), fabsf(c.y), fabsf(c.z)) + d); }
FCPWGB_D float bandRadius2(float d, float3 c) {
    float t = d + tieBand(c, d);
    return t * t;
}
template<bool TRACK> struct NearTie {  // off: no runner-up state, the same visiting radius
    FCPWGB_D float prune(float r2, float3 c) const { return bandRadius2(sqrtf(r2), c); }
    FCPWGB_D float pruneHit(float d, float3 c) const { return bandRadius2(d, c); }
    FCPWGB_D void replaced(float, uint32_t) {}
    FCPWGB_D void offer(float, uint32_t, uint32_t) {}
};
template<> struct NearTie<true> {  // two registers; the band is recomputed from the query when needed
    float d2nd = kFltMax;
    uint32_t sel2nd = kUintMax;
    FCPWGB_D float pruneHit(float d, float3 c) const { return bandRadius2(d, c); }
    FCPWGB_D float prune(float r2, float3 c) const { return bandRadius2(sqrtf(r2), c); }
    // the previous winner becomes the runner-up when a primitive beats it
    FCPWGB_D void replaced(float d, uint32_t sel) {
        d2nd = d;
        sel2nd = sel;
    }
    // a primitive that did not beat the winner (the caller's radius is checked
    // at the end); ranked like the winner, by distance and then leaf position.
    // The winner itself is not its own runner-up: the persistent schedule
    // tests its seed before the walk and meets it again in its leaf.
    FCPWGB_D void offer(float d, uint32_t sel, uint32_t winner) {
        if (sel != winner && (d < d2nd || (d == d2nd && sel < sel2nd))) {
            d2nd = d;
            sel2nd = sel;
        }
    }
};

// Whether a tested primitive (distance d, leaf position sel) becomes the
// winner: before the first hit when d*d <= r2 (the caller's radius, or a
// child's far distance); after it (r2 is then the winner's d*d) on a smaller
// distance, or on an equal one with an earlier leaf position. Boxes are
// visited within the winner's distance plus the rounding band (NearTie), so
// every primitive at the winner's distance is tested and an exact tie
// resolves to the same primitive in any visiting order: the result depends
// neither on the order of the queries, nor on which queries share a warp,
// nor on the wide layout. The runner-up of NearTie is ranked the same way.
FCPWGB_D bool beatsWinner(bool found, float d, float r2, float bestD, uint32_t sel, uint32_t selected) {
    return found ? (d < bestD || (d == bestD && sel < selected)) : d * d <= r2;
}

// A tested primitive becomes the winner: its distance always; its point, uv
// and index only where the traversal writes the record from them. In precise
// mode the record is formed from the winner's leaf position at the end (by
// the refinement pass on triangles, by finishQuery on segments), so the
// traversal keeps no point, uv or index (five registers fewer around the
// traversal loop, and the FP32 uv is never formed inside it).
template<class Prim, bool PRECISE> constexpr bool kKeepsRecord = !PRECISE;
template<class Prim, bool PRECISE>
FCPWGB_D void takeWinner(DevInteraction &best, float d, float3 pt, float2 uv, uint32_t index) {
    if constexpr (kKeepsRecord<Prim, PRECISE>) {
        best.p = pt;
        best.n = make_float3(0.f, 0.f, 0.f);
        best.uv = uv;
        best.index = index;
    }
    best.d = d;
}

// Closest point of one query on a wide tree (bvh.slang:395-502 semantics:
// inclusive d2Min <= r2 pruning, r2 shrunk by child d2Max, primitives accepted
// when d*d <= r2; exact distance ties go to the earlier leaf position, see
// beatsWinner).
// `root` is the tree's root record (always an inner record); `found`/`best`/
// `selected`/`r2` may arrive holding a candidate already tested (a seed).
// Boxes are pruned against rp2: r2, or with TRACK r2 widened by the band.
template<int W, int BITS, class Prim, bool TRACK, bool STATS, int SHORT>
FCPWGB_D bool wideClosest(const unsigned char *__restrict__ nodes, const unsigned char *__restrict__ prims,
                          uint32_t root, float3 c, float r2, bool found, DevInteraction &best, uint32_t &selected,
                          NearTie<TRACK> &tie, WideStack<SHORT> &st, uint32_t *errorWord, Count<STATS> &nExpanded,
                          Count<STATS> &nTests) {
    int sp = 0;
    uint32_t cur = root;
    WideNodeRegs<W, BITS> node;
    float rp2 = found ? tie.pruneHit(best.d, c) : tie.prune(r2, c);
    for (;;) {
        if (!(cur & kLeafBit)) {
            node.load(nodes, cur);
            nExpanded.add(1);
            constexpr uint32_t kSlotMask = W - 1;
            float d2Min[W];
            childD2Min<W, BITS>(node, c, d2Min);
            // a child's far distance bounds the answer; once a primitive has been
            // found r2 is a primitive distance and far distances rarely improve
            // it, so they are computed only before the first hit
            if (!found) {
#pragma unroll
                for (int k = 0; k < W; k++)
                    if (node.cnt(k) != kWideEmpty) r2 = fminf(r2, childD2Max<W, BITS>(node, c, k));
                rp2 = tie.prune(r2, c);
            }
            // keys: distance bits with the slot in the low bits, truncating the
            // distance downwards (visits are decided on d2Min <= rp2, so a smaller
            // stored distance can only add visits, never skip one)
            uint32_t key[W];
            int nh = 0;
#pragma unroll
            for (int k = 0; k < W; k++) {
                bool hit = node.cnt(k) != kWideEmpty && d2Min[k] <= rp2;
                key[k] = hit ? ((__float_as_uint(d2Min[k]) & ~kSlotMask) | (uint32_t)k) : 0xffffffffu;
                nh += hit ? 1 : 0;
            }
            sortNetwork<W>(key);
            if (nh > 0) {
                if (sp + nh - 1 > kWideStack) {
                    atomicOr(errorWord, kErrStackOverflow);
                    return found;
                }
                uint32_t firstRef = 0, refs[W];
                childRefs<W, BITS>(node, refs);
#pragma unroll
                for (int k = W - 1; k >= 0; k--) {
                    if (k < nh) {
                        uint32_t packed = selectBySlot<W>(refs, key[k] & kSlotMask);
                        if (k == 0) {
                            firstRef = packed;
                        } else {
                            st.push(sp, packed, __uint_as_float(key[k] & ~kSlotMask));
                            sp++;
                        }
                    }
                }
                cur = firstRef;
                continue;
            }
        } else {
            uint32_t off = cur & 0x07ffffffu, cnt = (cur >> 27) & 0xfu;
            nTests.add(cnt);
            for (uint32_t p = 0; p < cnt; p++) {
                Prim prim = Prim::load(prims, off + p);
                float3 pt;
                float2 uv;
                float d = prim.closestPoint(c, pt, uv);
                if (beatsWinner(found, d, r2, best.d, off + p, selected)) {
                    if (found) tie.replaced(best.d, selected);
                    r2 = fminf(r2, d * d);
                    rp2 = tie.pruneHit(d, c);
                    takeWinner<Prim, TRACK>(best, d, pt, uv, prim.index);
                    selected = off + p;
                    found = true;
                } else {
                    tie.offer(d, off + p, selected);
                }
            }
        }
        bool next = false;
        while (sp > 0) {
            sp--;
            if (st.dist(sp) <= rp2) {
                cur = st.ref(sp);
                next = true;
                break;
            }
        }
        if (!next) break;
    }
    return found;
}

// Precise record of a query from the traversal's winner (leaf position
// `first`; best holds its FP32 distance, uv and index) and runner-up within
// the rounding band and the caller's radius (`second`, FP32 distance
// dSecond; kUintMax: none): both refined (Prim::refine), the runner-up's
// record when it is closer by more than the refinement's own rounding (an
// exact tie -- two faces sharing the closest edge, whose formulas round
// differently -- stays with the winner, the earlier leaf position, so every
// layout and schedule returns the same record), and the face normal of the
// one kept (recordNormal).
template<class Prim>
FCPWGB_D void refineRecord(const unsigned char *__restrict__ prims, float3 c, uint32_t first, uint32_t second,
                           float dSecond, int recordNormal, DevInteraction &best) {
    Prim prim = Prim::load(prims, first);
    float3 p;
    DS d = prim.refine(c, best.d, p);
    if (second != kUintMax) {
        const Prim q = Prim::load(prims, second);
        float3 p2;
        const DS d2 = q.refine(c, dSecond, p2);
        if (dsSub(d, d2).hi > kRefineTie * d.hi) {
            float3 pt;
            float2 uv;
            q.closestPoint(c, pt, uv);
            d = d2;
            p = p2;
            best.uv = uv;
            best.index = q.index;
            prim = q;
        }
    }
    best.d = d.hi;
    best.p = p;
    if (recordNormal) best.n = prim.normal();
}

// Final step of query i. Without PRECISE: the FP32 record of the winner,
// with its face normal (recordNormal), to the caller's slot. With PRECISE
// and Prim::kRefinePass: only the leaf positions of the winner and of the
// runner-up to sel[i]; the refinement pass (kRefineClosest) then writes the
// record. With PRECISE otherwise: the refined record (refineRecord).
template<class Prim, bool PRECISE>
FCPWGB_D void finishQuery(const unsigned char *__restrict__ prims, const uint32_t *__restrict__ perm,
                          DevInteraction *__restrict__ out, uint2 *__restrict__ sel, uint32_t i, float3 c,
                          float r2User, bool found, uint32_t selected, int recordNormal, DevInteraction &best,
                          const NearTie<PRECISE> &tie) {
    if constexpr (PRECISE) {
        const bool second = found && tie.sel2nd != kUintMax && tie.d2nd <= best.d + tieBand(c, best.d) &&
                            tie.d2nd * tie.d2nd <= r2User;
        if constexpr (Prim::kRefinePass) {
            sel[i] = make_uint2(found ? selected : kUintMax, second ? tie.sel2nd : kUintMax);
            return;
        } else if (found) {
            // the winner's uv and index, not kept by the traversal (takeWinner)
            const Prim w = Prim::load(prims, selected);
            float3 pt;
            w.closestPoint(c, pt, best.uv);
            best.index = w.index;
            refineRecord<Prim>(prims, c, selected, second ? tie.sel2nd : kUintMax, tie.d2nd, recordNormal, best);
        }
    } else {
        if (found && recordNormal) best.n = Prim::load(prims, selected).normal();
    }
    out[perm ? __ldg(perm + i) : i] = best;
}

// The precise record of a query at c from its winner (leaf position
// `first`) and runner-up within the band (`second`, kUintMax: none), each
// evaluated in FP32 (closest point for uv, distance as the refinement's
// conditioning estimate) and refined (Prim::refine); the runner-up's record
// replaces the winner's when its refined distance is smaller by more than
// kRefineTie, the same decision as refineRecord. One loop iteration per
// candidate keeps a single copy of the FP32 and double-single code in the
// kernel, whose warps otherwise stalled on instruction fetch.
template<class Prim>
FCPWGB_D DevInteraction refineCandidates(const unsigned char *__restrict__ prims, float3 c, uint32_t first,
                                         uint32_t second, int recordNormal) {
    DevInteraction best = defaultInteraction();
    DS dKeep = dsOf(kFltMax);
    uint32_t kept = first;
#pragma unroll 1
    for (int k = 0; k < 2; k++) {
        const uint32_t pos = k == 0 ? first : second;
        if (pos == kUintMax) break;
        const Prim prim = Prim::load(prims, pos);
        float3 pt, p;
        float2 uv;
        const float d32 = prim.closestPoint(c, pt, uv);
        const DS d = prim.refine(c, d32, p);
        if (k == 0 || dsSub(dKeep, d).hi > kRefineTie * dKeep.hi) {
            dKeep = d;
            kept = pos;
            best.p = p;
            best.uv = uv;
            best.index = prim.index;
        }
    }
    best.d = dKeep.hi;
    if (recordNormal) best.n = Prim::load(prims, kept).normal();
    return best;
}

// The refinement pass's work for sorted query i: refineCandidates on the
// leaf positions in sel[i], written to the caller's slot; without a winner,
// the default record.
template<class Prim>
FCPWGB_D void refineQuery(const unsigned char *__restrict__ prims, const DevSphere *__restrict__ spheres,
                          const uint32_t *__restrict__ perm, const uint2 *__restrict__ sel,
                          DevInteraction *__restrict__ out, uint32_t i, int recordNormal) {
    const uint2 s = __ldg(sel + i);
    DevInteraction best = defaultInteraction();
    if (s.x != kUintMax) {
        const float4 s4 = ldg4(spheres + i);
        best = refineCandidates<Prim>(prims, make_float3(s4.x, s4.y, s4.z), s.x, s.y, recordNormal);
    }
    out[perm ? __ldg(perm + i) : i] = best;
}

// One thread per query. With `perm` non-NULL the queries are read in sorted
// order and results scattered back to out[perm[i]]; with `roots` non-NULL
// query i starts at wide record roots[i] (a forest of trees), else at 0; with
// `stats` non-NULL expansions and primitive tests are summed into stats[1..2].
// With `counter` non-NULL the blocks are persistent: a warp takes kWidePool
// consecutive (sorted, so neighbouring) queries at a time from the counter and
// walks them in rounds of 32, and a lane's previous winner -- a primitive
// near its next query -- is tested first, so that query starts with a tight
// radius instead of FLT_MAX. Any tested primitive is a valid candidate, so the
// result is the same closest distance (ties may pick another primitive).
constexpr uint32_t kWidePool = 256;
template<int W, int BITS, class Prim, bool PRECISE, bool PERSISTENT, bool STATS, int SHORT>
__global__ void __launch_bounds__(kWideBlock, 8) kWideClosestPoint(const unsigned char *__restrict__ nodes,
                                                                const unsigned char *__restrict__ prims,
                                                                const DevSphere *__restrict__ spheres,
                                                                const uint32_t *__restrict__ perm,
                                                                const uint32_t *__restrict__ roots,
                                                                DevInteraction *__restrict__ out,
                                                                uint2 *__restrict__ sel, uint32_t n,
                                                                int recordNormal, uint32_t *counter,
                                                                uint32_t *errorWord, unsigned long long *stats) {
    __shared__ uint32_t sRef[SHORT > 0 ? SHORT * kWideBlock : 1];
    __shared__ float sD[SHORT > 0 ? SHORT * kWideBlock : 1];
    WideStack<SHORT> st;
    st.sRef = sRef + threadIdx.x;
    st.sD = sD + threadIdx.x;
    Count<STATS> tExp, tTests;
    if (!PERSISTENT) {
        uint32_t i = blockIdx.x * kWideBlock + threadIdx.x;
        if (i < n) {
            float4 s4 = ldg4(spheres + i);
            float3 c = make_float3(s4.x, s4.y, s4.z);
            DevInteraction best = defaultInteraction();
            uint32_t selected = kUintMax;
            uint32_t root = roots ? __ldg(roots + i) : 0u;
            NearTie<PRECISE> tie;
            const float r2 = queryRadius2(c, s4.w);
            bool found = wideClosest<W, BITS, Prim, PRECISE, STATS, SHORT>(nodes, prims, root, c, r2, false, best, selected, tie,
                                                             st, errorWord, tExp, tTests);
            finishQuery<Prim, PRECISE>(prims, perm, out, sel, i, c, r2, found, selected, recordNormal, best, tie);
        }
    } else {
        const uint32_t lane = threadIdx.x & 31u;
        for (;;) {
            __syncwarp();
            uint32_t b = 0;
            if (lane == 0) b = atomicAdd(counter, kWidePool);
            b = __shfl_sync(0xffffffffu, b, 0);
            if (b >= n) break;
            const uint32_t e = min(b + kWidePool, n);
            uint32_t seed = kUintMax, seedRoot = kUintMax;
            for (uint32_t i = b + lane; i < e; i += 32) {
                float4 s4 = ldg4(spheres + i);
                float3 c = make_float3(s4.x, s4.y, s4.z);
                float r2 = queryRadius2(c, s4.w);
                const float r2User = r2;
                DevInteraction best = defaultInteraction();
                uint32_t selected = kUintMax;
                uint32_t root = roots ? __ldg(roots + i) : 0u;
                bool found = false;
                NearTie<PRECISE> tie;
                if (seed != kUintMax && seedRoot == root) {
                    Prim prim = Prim::load(prims, seed);
                    float3 pt;
                    float2 uv;
                    float d = prim.closestPoint(c, pt, uv);
                    tTests.add(1);
                    if (d * d <= r2) {
                        r2 = d * d;
                        takeWinner<Prim, PRECISE>(best, d, pt, uv, prim.index);
                        selected = seed;
                        found = true;
                    }
                }
                found = wideClosest<W, BITS, Prim, PRECISE, STATS, SHORT>(nodes, prims, root, c, r2, found, best, selected, tie,
                                                            st, errorWord, tExp, tTests);
                seed = found ? selected : kUintMax;
                seedRoot = root;
                finishQuery<Prim, PRECISE>(prims, perm, out, sel, i, c, r2User, found, selected, recordNormal, best, tie);
            }
        }
    }
    if (STATS && stats) {
        atomicAdd(stats + 1, tExp.get());
        atomicAdd(stats + 2, tTests.get());
    }
}

// Packet traversal: the 32 (sorted, neighbouring) queries of a warp walk the
// tree together. Each visited record is loaded once for the warp (all lanes
// read the same address) and every lane tests its own query against it; a
// lane takes part in a record only while the record's box is within its own
// search radius, so each query still prunes exactly as alone. A child is
// visited when any lane needs it (a ballot), in the order of one lane's
// distances; per-lane child distances stay on a warp stack (shared memory,
// one column per lane) and are re-checked against each lane's radius when the
// entry is popped. Queries of a warp that start at different roots (a forest
// whose scene boundary falls inside the warp) are walked one root at a time.
constexpr int kPacketShort = 32;  // warp-stack entries held in shared memory
// With `counter` non-NULL the blocks are persistent (one resident wave) and
// every warp takes its next packet -- 32 consecutive sorted queries -- from
// the counter as soon as its previous one is done, so a block whose warps
// finish unevenly keeps all of them busy instead of holding its slot until
// the slowest warp ends.
template<int W, int BITS, class Prim, bool PRECISE, bool STATS>
__global__ void __launch_bounds__(kWideBlock, 8) kWidePacketClosestPoint(const unsigned char *__restrict__ nodes,
                                                                      const unsigned char *__restrict__ prims,
                                                                      const DevSphere *__restrict__ spheres,
                                                                      const uint32_t *__restrict__ perm,
                                                                      const uint32_t *__restrict__ roots,
                                                                      DevInteraction *__restrict__ out,
                                                                      uint2 *__restrict__ sel, uint32_t n,
                                                                      int recordNormal, uint32_t *counter,
                                                                      uint32_t *errorWord,
                                                                      unsigned long long *stats) {
    constexpr uint32_t kSlotMask = W - 1;
    constexpr int kWarps = kWideBlock / 32;
    __shared__ uint32_t sRef[kWarps][kPacketShort];
    __shared__ float sDist[kWarps][kPacketShort][32];
    uint32_t lRef[kWideStack - kPacketShort];  // deeper entries: every lane keeps the (uniform) refs
    float lDist[kWideStack - kPacketShort];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    Count<STATS> tExp, tTests, tVisits, tPrimLoads;
    WideNodeRegs<W, BITS> node;
    uint32_t i = blockIdx.x * kWideBlock + threadIdx.x;
    for (;;) {
        if (counter) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(counter, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n) break;
            i = base + lane;
        }
        const bool valid = i < n;
        float3 c = make_float3(0.f, 0.f, 0.f);
        float r2 = -1.0f;  // a lane without a query needs nothing
        uint32_t root = 0;
        if (valid) {
            float4 s4 = ldg4(spheres + i);
            c = make_float3(s4.x, s4.y, s4.z);
            r2 = queryRadius2(c, s4.w);
            root = roots ? __ldg(roots + i) : 0u;
        }
        DevInteraction best = defaultInteraction();
        uint32_t selected = kUintMax;
        bool found = false;
        NearTie<PRECISE> tie;
        const float r2User = r2;
        float rp2 = tie.prune(r2, c);  // pruning radius^2 (NaN for a lane without a query)

        uint32_t pending = __ballot_sync(0xffffffffu, valid);
        while (pending) {
            const uint32_t rootNow = __shfl_sync(0xffffffffu, root, __ffs(pending) - 1);
            const bool mine = valid && root == rootNow && ((pending >> lane) & 1u);
            pending &= ~__ballot_sync(0xffffffffu, mine);
            bool act = mine;  // this lane needs the current record
            uint32_t cur = rootNow;
            int sp = 0;       // warp-uniform
            for (;;) {
                bool descend = false;
                if (!(cur & kLeafBit)) {
                    node.load(nodes, cur);
                    tVisits.add(1);
                    float d2Min[W];
                    childD2Min<W, BITS>(node, c, d2Min);
                    if (act) tExp.add(1);
                    // no far-distance shrink of r2 before the first hit (the reference's
                    // d2Max, which one thread per query keeps): the packet descends in its
                    // first lane's nearest-first order anyway, lanes meet primitives within a
                    // few records, and the W far distances per record cost more issue slots
                    // than the pruning saved (6.69 to 6.36 ms on 4M queries, same records:
                    // the winner does not depend on the radius a query starts from)
                    // children needed by any lane (one OR over the warp of each lane's
                    // mask), ordered by the first active lane's distances
                    uint32_t needMask = 0;
#pragma unroll
                    for (int k = 0; k < W; k++)
                        needMask |= (act && node.cnt(k) != kWideEmpty && d2Min[k] <= rp2) ? (1u << k) : 0u;
                    const uint32_t anyMask = __reduce_or_sync(0xffffffffu, needMask);
                    const uint32_t leader = __ffs(__ballot_sync(0xffffffffu, act)) - 1;
                    uint32_t key[W];
#pragma unroll
                    for (int k = 0; k < W; k++) {
                        const float lead = __shfl_sync(0xffffffffu, d2Min[k], leader);
                        key[k] = ((anyMask >> k) & 1u) ? ((__float_as_uint(lead) & ~kSlotMask) | (uint32_t)k) : 0xffffffffu;
                    }
                    const int nh = __popc(anyMask);
                    sortNetwork<W>(key);
                    if (nh > 0) {
                        if (sp + nh - 1 > kWideStack) {
                            if (lane == 0) atomicOr(errorWord, kErrStackOverflow);
                            break;
                        }
                        uint32_t rawRefs[W];
#pragma unroll
                        for (int s = 0; s < W; s++) rawRefs[s] = node.ref(s);
#pragma unroll
                        for (int k = W - 1; k >= 0; k--) {
                            if (k < nh) {
                                const uint32_t slot = key[k] & kSlotMask;
                                const uint32_t cnt = node.cntAt(slot);
                                const uint32_t ref = selectBySlot<W>(rawRefs, slot);
                                const uint32_t packed = cnt == 0 ? ref : packLeaf(ref, cnt);
                                // a lane out of this record is out of its children too (NaN is never <= rp2)
                                const float dl = act ? selectBySlot<W>(d2Min, slot) : __int_as_float(0x7fc00000);
                                if (k == 0) {
                                    cur = packed;
                                    act = dl <= rp2;
                                } else {
                                    if (sp < kPacketShort) {
                                        if (lane == 0) sRef[warp][sp] = packed;
                                        sDist[warp][sp][lane] = dl;
                                    } else {
                                        lRef[sp - kPacketShort] = packed;
                                        lDist[sp - kPacketShort] = dl;
                                    }
                                    sp++;
                                }
                            }
                        }
                        __syncwarp();
                        descend = true;
                    }
                } else {
                    uint32_t off = cur & 0x07ffffffu, cnt = (cur >> 27) & 0xfu;
                    tPrimLoads.add(cnt);
                    if (act) tTests.add(cnt);
                    for (uint32_t p = 0; p < cnt; p++) {
                        Prim prim = Prim::load(prims, off + p);
                        if (act) {
                            float3 pt;
                            float2 uv;
                            float d = prim.closestPoint(c, pt, uv);
                            if (beatsWinner(found, d, r2, best.d, off + p, selected)) {
                                if (found) tie.replaced(best.d, selected);
                                r2 = fminf(r2, d * d);
                                rp2 = tie.pruneHit(d, c);
                                takeWinner<Prim, PRECISE>(best, d, pt, uv, prim.index);
                                selected = off + p;
                                found = true;
                            } else {
                                tie.offer(d, off + p, selected);
                            }
                        }
                    }
                }
                if (descend) continue;
                // pop until some lane needs the entry
                bool next = false;
                while (sp > 0) {
                    sp--;
                    uint32_t ref;
                    float dl;
                    if (sp < kPacketShort) {
                        ref = sRef[warp][sp];
                        dl = sDist[warp][sp][lane];
                    } else {
                        ref = lRef[sp - kPacketShort];
                        dl = lDist[sp - kPacketShort];
                    }
                    act = dl <= rp2;
                    if (__ballot_sync(0xffffffffu, act)) {
                        cur = ref;
                        next = true;
                        break;
                    }
                }
                __syncwarp();
                if (!next) break;
            }
        }
        if (valid) finishQuery<Prim, PRECISE>(prims, perm, out, sel, i, c, r2User, found, selected, recordNormal, best, tie);
        if (!counter) break;
    }
    if (STATS && stats) {
        if (lane == 0) {
            atomicAdd(stats + 3, tVisits.get());
            atomicAdd(stats + 4, tPrimLoads.get());
        }
        atomicAdd(stats + 1, tExp.get());
        atomicAdd(stats + 2, tTests.get());
    }
}

}  // namespace fcpwgb
#include "k_wide_coop.cuh"
namespace fcpwgb {

// Ray first hit / occlusion on a wide tree, one thread per ray, with the
// semantics of bvh.slang:144-254: a child is entered when the slab test with
// the parallel-slab guard passes against the current tMax, nearest entry
// first; a stacked child is skipped when its entry distance exceeds tMax;
// hits are accepted when 0 <= t <= tMax (a later equal t wins), and an
// occlusion query stops at its first hit.
// Ray traversal of one wide tree from record `root` (the loop of kWideRay);
// r.tMax shrinks to the nearest hit, `best` receives it. Returns whether the
// ray hit (with occl: whether it is occluded; only best.index is set then).
template<int W, int BITS, class Prim, int SHORT>
FCPWGB_D bool wideRay(const unsigned char *__restrict__ nodes, const unsigned char *__restrict__ prims,
                      uint32_t root, DevRay &r, int occl, DevInteraction &best, WideStack<SHORT> &st,
                      uint32_t *errorWord, uint32_t &tExp, uint32_t &tTests) {
    constexpr uint32_t kSlotMask = W - 1;
    bool anyHit = false;
    WideNodeRegs<W, BITS> node;
    uint32_t cur = root;
    int sp = 0;
    bool done = false;
    while (!done) {
        if (!(cur & kLeafBit)) {
            node.load(nodes, cur);
            tExp++;
            uint32_t key[W];
            int nh = 0;
#pragma unroll
            for (int k = 0; k < W; k++) {
                float t0, t1;
                bool hit = node.cnt(k) != kWideEmpty &&
                           boxRayIntersect(make_float3(node.bound(0, k), node.bound(1, k), node.bound(2, k)),
                                           make_float3(node.bound(3, k), node.bound(4, k), node.bound(5, k)), r, t0,
                                           t1);
                // entry distances are >= 0 (+ 0 turns a -0 into +0), so their bits sort as integers
                key[k] = hit ? ((__float_as_uint(t0 + 0.0f) & ~kSlotMask) | (uint32_t)k) : 0xffffffffu;
                nh += hit ? 1 : 0;
            }
            sortNetwork<W>(key);
            if (nh > 0) {
                if (sp + nh - 1 > kWideStack) {
                    atomicOr(errorWord, kErrStackOverflow);
                    break;
                }
                uint32_t refs[W];
                childRefs<W, BITS>(node, refs);
#pragma unroll
                for (int k = W - 1; k >= 1; k--) {
                    if (k < nh) {
                        st.push(sp, selectBySlot<W>(refs, key[k] & kSlotMask), __uint_as_float(key[k] & ~kSlotMask));
                        sp++;
                    }
                }
                cur = selectBySlot<W>(refs, key[0] & kSlotMask);
                continue;
            }
        } else {
            uint32_t off = cur & 0x07ffffffu, cnt = (cur >> 27) & 0xfu;
            tTests += cnt;
            for (uint32_t p = 0; p < cnt; p++) {
                Prim prim = Prim::load(prims, off + p);
                DevInteraction c = defaultInteraction();
                if (prim.intersect(r, occl != 0, c)) {
                    c.index = prim.index;
                    anyHit = true;
                    if (occl) {
                        best.index = c.index;
                        done = true;
                        break;
                    }
                    r.tMax = fminf(r.tMax, c.d);
                    best = c;
                }
            }
            if (done) break;
        }
        bool next = false;
        while (sp > 0) {
            sp--;
            if (st.dist(sp) <= r.tMax) {
                cur = st.ref(sp);
                next = true;
                break;
            }
        }
        if (!next) break;
    }
    return anyHit;
}

template<int W, int BITS, class Prim>
__global__ void __launch_bounds__(kWideBlock, 8) kWideRay(const unsigned char *__restrict__ nodes,
                                                       const unsigned char *__restrict__ prims,
                                                       const DevRay *__restrict__ rays,
                                                       const uint32_t *__restrict__ perm,
                                                       DevInteraction *__restrict__ out, uint32_t n, int occl,
                                                       const DevRay *__restrict__ callerRays, const int *sortInfo,
                                                       uint32_t *errorWord, unsigned long long *stats) {
    // rays the sort left in the caller's order are read from the caller's array
    if (sortInfo && keepOrder(sortInfo, n)) {
        rays = callerRays;
        perm = nullptr;
    }
    __shared__ uint32_t sRef[kShortStack * kWideBlock];
    __shared__ float sD[kShortStack * kWideBlock];
    WideStack<kShortStack> st;
    st.sRef = sRef + threadIdx.x;
    st.sD = sD + threadIdx.x;
    const uint32_t i = blockIdx.x * kWideBlock + threadIdx.x;
    if (i >= n) return;
    const unsigned char *rp = reinterpret_cast<const unsigned char *>(rays + i);
    float2 a = ldg2(rp), b = ldg2(rp + 8), cc = ldg2(rp + 16), d = ldg2(rp + 24), e = ldg2(rp + 32);
    DevRay r;
    r.o = make_float3(a.x, a.y, b.x);
    r.d = make_float3(b.y, cc.x, cc.y);
    r.dInv = make_float3(d.x, d.y, e.x);
    r.tMax = e.y;
    DevInteraction best = defaultInteraction();
    uint32_t tExp = 0, tTests = 0;
    wideRay<W, BITS, Prim, kShortStack>(nodes, prims, 0u, r, occl, best, st, errorWord, tExp, tTests);
    out[perm ? __ldg(perm + i) : i] = best;
    if (stats) {
        atomicAdd(stats + 1, (unsigned long long)tExp);
        atomicAdd(stats + 2, (unsigned long long)tTests);
    }
}

// Rays with per-lane refill (persistent blocks, one resident wave): a lane
// whose ray is finished takes the next one at once (one atomicAdd per warp for
// all lanes that need a ray), and every iteration advances each active lane's
// ray by one step -- one record (child slab tests, nearest entry next, the
// others pushed farthest first) or one leaf (its primitives, then a pop) -- so
// lanes stay busy however unequal the rays' traversals are (most random rays
// leave the scene box after a few records, a few cross many). The semantics
// are those of wideRay: children within the current tMax, stacked entries
// skipped once beyond it, hits accepted when 0 <= t <= tMax (a later equal t
// wins), an occlusion ray done at its first hit. Only the winner's leaf
// position is kept during the walk; its record (point, normal, uv) is
// recomputed from it at the end with the same arithmetic.
template<int W, int BITS, class Prim>
__global__ void __launch_bounds__(kWideBlock, 8) kWideRayRefill(const unsigned char *__restrict__ nodes,
                                                             const unsigned char *__restrict__ prims,
                                                             const DevRay *__restrict__ rays,
                                                             const uint32_t *__restrict__ perm,
                                                             DevInteraction *__restrict__ out, uint32_t n, int occl,
                                                             const DevRay *__restrict__ callerRays,
                                                             const int *sortInfo, uint32_t *counter,
                                                             uint32_t *errorWord, unsigned long long *stats) {
    constexpr uint32_t kSlotMask = W - 1;
    if (sortInfo && keepOrder(sortInfo, n)) {  // rays left in the caller's order
        rays = callerRays;
        perm = nullptr;
    }
    __shared__ uint32_t sRef[kShortStack * kWideBlock];
    __shared__ float sD[kShortStack * kWideBlock];
    WideStack<kShortStack> st;
    st.sRef = sRef + threadIdx.x;
    st.sD = sD + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    bool active = false;
    uint32_t id = 0, cur = 0, bestSel = kUintMax;
    int sp = 0;
    DevRay r;
    unsigned long long tExp = 0, tTests = 0;
    WideNodeRegs<W, BITS> node;
    for (;;) {
        const uint32_t need = __ballot_sync(0xffffffffu, !active);
        if (need) {
            const uint32_t leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active) {
                id = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
                if (id < n) {
                    const unsigned char *rp = reinterpret_cast<const unsigned char *>(rays + id);
                    const float2 a = ldg2(rp), b = ldg2(rp + 8), cc = ldg2(rp + 16), d = ldg2(rp + 24),
                                 e = ldg2(rp + 32);
                    r.o = make_float3(a.x, a.y, b.x);
                    r.d = make_float3(b.y, cc.x, cc.y);
                    r.dInv = make_float3(d.x, d.y, e.x);
                    r.tMax = e.y;
                    cur = 0;
                    sp = 0;
                    bestSel = kUintMax;
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (!active) continue;
        bool popNext = true, finished = false;
        if (!(cur & kLeafBit)) {
            node.load(nodes, cur);
            tExp++;
            uint32_t key[W];
            int nh = 0;
#pragma unroll
            for (int k = 0; k < W; k++) {
                float t0, t1;
                const bool hit = node.cnt(k) != kWideEmpty &&
                                 boxRayIntersect(make_float3(node.bound(0, k), node.bound(1, k), node.bound(2, k)),
                                                 make_float3(node.bound(3, k), node.bound(4, k), node.bound(5, k)), r,
                                                 t0, t1);
                key[k] = hit ? ((__float_as_uint(t0 + 0.0f) & ~kSlotMask) | (uint32_t)k) : 0xffffffffu;
                nh += hit ? 1 : 0;
            }
            sortNetwork<W>(key);
            if (nh > 0) {
                if (sp + nh - 1 > kWideStack) {
                    atomicOr(errorWord, kErrStackOverflow);
                    finished = true;
                } else {
                    uint32_t refs[W];
                    childRefs<W, BITS>(node, refs);
#pragma unroll
                    for (int k = W - 1; k >= 1; k--) {
                        if (k < nh) {
                            st.push(sp, selectBySlot<W>(refs, key[k] & kSlotMask),
                                    __uint_as_float(key[k] & ~kSlotMask));
                            sp++;
                        }
                    }
                    cur = selectBySlot<W>(refs, key[0] & kSlotMask);
                    popNext = false;
                }
            }
        } else {
            const uint32_t off = cur & 0x07ffffffu, cnt = (cur >> 27) & 0xfu;
            tTests += cnt;
            for (uint32_t p = 0; p < cnt; p++) {
                const Prim prim = Prim::load(prims, off + p);
                DevInteraction c;
                if (prim.intersect(r, occl != 0, c)) {
                    bestSel = off + p;
                    if (occl) {
                        finished = true;
                        break;
                    }
                    r.tMax = fminf(r.tMax, c.d);
                }
            }
        }
        if (popNext && !finished) {
            finished = true;
            while (sp > 0) {
                sp--;
                if (st.dist(sp) <= r.tMax) {
                    cur = st.ref(sp);
                    finished = false;
                    break;
                }
            }
        }
        if (finished) {
            DevInteraction best = defaultInteraction();
            if (bestSel != kUintMax) {
                const Prim prim = Prim::load(prims, bestSel);
                if (!occl) prim.intersect(r, false, best);  // the winner again: r.tMax is its t
                best.index = prim.index;
            }
            out[perm ? __ldg(perm + id) : id] = best;
            active = false;
        }
    }
    if (stats) {
        atomicAdd(stats + 1, tExp);
        atomicAdd(stats + 2, tTests);
    }
}

// Ray packets: the 32 (sorted) rays of a warp walk the wide tree together,
// as kWidePacketClosestPoint does for closest points. Each record is loaded
// once for the warp; every lane slab-tests its own ray against every child
// (within its own tMax) and takes part in a child only while the child's
// entry distance is within its tMax, re-checked when the entry is popped;
// children go in the order of the first active lane's entry distances. A
// hit shrinks the lane's tMax; an occlusion ray leaves the packet at its
// first hit. Rays sorted by direction octant and origin keep the lanes'
// paths alike.
template<int W, int BITS, class Prim>
__global__ void __launch_bounds__(kWideBlock, 8) kWidePacketRay(const unsigned char *__restrict__ nodes,
                                                             const unsigned char *__restrict__ prims,
                                                             const DevRay *__restrict__ rays,
                                                             const uint32_t *__restrict__ perm,
                                                             DevInteraction *__restrict__ out, uint32_t n, int occl,
                                                             const DevRay *__restrict__ callerRays,
                                                             const int *sortInfo, uint32_t *errorWord,
                                                             unsigned long long *stats) {
    if (sortInfo && keepOrder(sortInfo, n)) {  // rays left in the caller's order
        rays = callerRays;
        perm = nullptr;
    }
    constexpr uint32_t kSlotMask = W - 1;
    constexpr int kWarps = kWideBlock / 32;
    __shared__ uint32_t sRef[kWarps][kPacketShort];
    __shared__ float sDist[kWarps][kPacketShort][32];
    uint32_t lRef[kWideStack - kPacketShort];
    float lDist[kWideStack - kPacketShort];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t i = blockIdx.x * kWideBlock + threadIdx.x;
    const bool valid = i < n;
    DevRay r;
    r.o = r.d = r.dInv = make_float3(0.0f, 0.0f, 0.0f);
    r.tMax = -1.0f;  // a lane without a ray needs nothing
    if (valid) {
        const unsigned char *rp = reinterpret_cast<const unsigned char *>(rays + i);
        float2 a = ldg2(rp), b = ldg2(rp + 8), cc = ldg2(rp + 16), d = ldg2(rp + 24), e = ldg2(rp + 32);
        r.o = make_float3(a.x, a.y, b.x);
        r.d = make_float3(b.y, cc.x, cc.y);
        r.dInv = make_float3(d.x, d.y, e.x);
        r.tMax = e.y;
    }
    DevInteraction best = defaultInteraction();
    uint32_t tExp = 0, tTests = 0;
    WideNodeRegs<W, BITS> node;
    bool act = valid;
    uint32_t cur = 0;
    int sp = 0;  // warp-uniform
    if (__ballot_sync(0xffffffffu, act)) {
        for (;;) {
            bool descend = false;
            if (!(cur & kLeafBit)) {
                node.load(nodes, cur);
                if (act) tExp++;
                float t0[W];
                uint32_t needMask = 0;
#pragma unroll
                for (int k = 0; k < W; k++) {
                    float a0, a1;
                    const bool hit =
                        act && node.cnt(k) != kWideEmpty &&
                        boxRayIntersect(make_float3(node.bound(0, k), node.bound(1, k), node.bound(2, k)),
                                        make_float3(node.bound(3, k), node.bound(4, k), node.bound(5, k)), r, a0, a1);
                    // entry distances are >= 0 (+ 0 turns a -0 into +0); NaN where this lane misses
                    t0[k] = hit ? a0 + 0.0f : __int_as_float(0x7fc00000);
                    needMask |= hit ? (1u << k) : 0u;
                }
                const uint32_t anyMask = __reduce_or_sync(0xffffffffu, needMask);
                const uint32_t leader = __ffs(__ballot_sync(0xffffffffu, act)) - 1;
                uint32_t key[W];
#pragma unroll
                for (int k = 0; k < W; k++) {
                    // a child the leader misses sorts after the ones it enters (NaN bits)
                    const float lead = __shfl_sync(0xffffffffu, t0[k], leader);
                    key[k] = ((anyMask >> k) & 1u) ? ((__float_as_uint(lead) & ~kSlotMask) | (uint32_t)k) : 0xffffffffu;
                }
                const int nh = __popc(anyMask);
                sortNetwork<W>(key);
                if (nh > 0) {
                    if (sp + nh - 1 > kWideStack) {
                        if (lane == 0) atomicOr(errorWord, kErrStackOverflow);
                        break;
                    }
                    uint32_t rawRefs[W];
#pragma unroll
                    for (int s = 0; s < W; s++) rawRefs[s] = node.ref(s);
#pragma unroll
                    for (int k = W - 1; k >= 0; k--) {
                        if (k < nh) {
                            const uint32_t slot = key[k] & kSlotMask;
                            const uint32_t cnt = node.cntAt(slot);
                            const uint32_t ref = selectBySlot<W>(rawRefs, slot);
                            const uint32_t packed = cnt == 0 ? ref : packLeaf(ref, cnt);
                            const float dl = selectBySlot<W>(t0, slot);
                            if (k == 0) {
                                cur = packed;
                                act = dl <= r.tMax;
                            } else {
                                if (sp < kPacketShort) {
                                    if (lane == 0) sRef[warp][sp] = packed;
                                    sDist[warp][sp][lane] = dl;
                                } else {
                                    lRef[sp - kPacketShort] = packed;
                                    lDist[sp - kPacketShort] = dl;
                                }
                                sp++;
                            }
                        }
                    }
                    __syncwarp();
                    descend = true;
                }
            } else {
                const uint32_t off = cur & 0x07ffffffu, cnt = (cur >> 27) & 0xfu;
                if (act) tTests += cnt;
                for (uint32_t p = 0; p < cnt; p++) {
                    const Prim prim = Prim::load(prims, off + p);
                    if (act) {
                        DevInteraction c = defaultInteraction();
                        if (prim.intersect(r, occl != 0, c)) {
                            c.index = prim.index;
                            if (occl) {
                                best.index = c.index;
                                act = false;
                                r.tMax = -1.0f;  // done: no entry is within it
                            } else {
                                r.tMax = fminf(r.tMax, c.d);
                                best = c;
                            }
                        }
                    }
                }
            }
            if (descend) continue;
            // pop until some lane needs the entry
            bool next = false;
            while (sp > 0) {
                sp--;
                uint32_t ref;
                float dl;
                if (sp < kPacketShort) {
                    ref = sRef[warp][sp];
                    dl = sDist[warp][sp][lane];
                } else {
                    ref = lRef[sp - kPacketShort];
                    dl = lDist[sp - kPacketShort];
                }
                act = dl <= r.tMax;
                if (__ballot_sync(0xffffffffu, act)) {
                    cur = ref;
                    next = true;
                    break;
                }
            }
            __syncwarp();
            if (!next) break;
        }
    }
    if (valid) out[perm ? __ldg(perm + i) : i] = best;
    if (stats && valid) {
        atomicAdd(stats + 1, (unsigned long long)tExp);
        atomicAdd(stats + 2, (unsigned long long)tTests);
    }
}

// Re-quantises every wide node from the (refit) binary boxes behind its slots.
template<int W, int BITS>
__global__ void kRequantize(unsigned char *wideNodes, const int32_t *childBinary, const unsigned char *binNodes,
                            int binStride, uint32_t nWide, uint32_t *errorWord) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nWide) return;
    float lo[W * 3], hi[W * 3];
    bool valid[W];
    for (int c = 0; c < W; c++) {
        int32_t b = childBinary[(size_t)i * W + c];
        valid[c] = b >= 0;
        for (int a = 0; a < 3; a++) { lo[c * 3 + a] = 0.0f; hi[c * 3 + a] = 0.0f; }
        if (b >= 0) {
            const float *f = reinterpret_cast<const float *>(binNodes + (size_t)b * binStride);
            for (int a = 0; a < 3; a++) { lo[c * 3 + a] = f[a]; hi[c * 3 + a] = f[3 + a]; }
        }
    }
    unsigned char rec[WideLayout<W, BITS>::kSize];
    unsigned char *dst = wideNodes + (size_t)i * WideLayout<W, BITS>::kSize;
    for (int k = 0; k < WideLayout<W, BITS>::kSize; k++) rec[k] = dst[k];
    if (!quantizeWideNode<W, BITS>(lo, hi, valid, rec)) {
        atomicOr(errorWord, kErrBadIndex);
        return;
    }
    for (int k = 0; k < WideLayout<W, BITS>::kSize; k++) dst[k] = rec[k];
}

template<int W, int B, class Prim, bool PRECISE, bool STATS, int L>
void launchCoop(const WideLaunch &l, cudaStream_t s) {
    constexpr uint32_t perBlock = kWideBlock / L;
    kWideCoopClosestPoint<W, B, Prim, PRECISE, STATS, L><<<dim3((l.n + perBlock - 1) / perBlock), dim3(kWideBlock),
                                                          0, s>>>(l.nodes, l.prims, l.spheres, l.perm, l.roots, l.out,
                                                                  l.sel, l.n, l.recordNormal, l.errorWord, l.stats);
}

template<int W, int B, class Prim, bool PRECISE, bool STATS>
cudaError_t launchWideClosestKernel(const WideLaunch &l, cudaStream_t s) {
    dim3 g(l.grid), b(kWideBlock);
    if (l.lanes == 2)
        launchCoop<W, B, Prim, PRECISE, STATS, 2>(l, s);
    else if (l.lanes == 4)
        launchCoop<W, B, Prim, PRECISE, STATS, 4>(l, s);
    else if (l.lanes == 8)
        launchCoop<W, B, Prim, PRECISE, STATS, 8>(l, s);
    else if (l.packet)
        kWidePacketClosestPoint<W, B, Prim, PRECISE, STATS><<<g, b, 0, s>>>(
            l.nodes, l.prims, l.spheres, l.perm, l.roots, l.out, l.sel, l.n, l.recordNormal, l.counter, l.errorWord,
            l.stats);
    else if (l.counter) {
        if (l.shortStack)
            kWideClosestPoint<W, B, Prim, PRECISE, true, STATS, kShortStack><<<g, b, 0, s>>>(
                l.nodes, l.prims, l.spheres, l.perm, l.roots, l.out, l.sel, l.n, l.recordNormal, l.counter, l.errorWord,
                l.stats);
        else
            kWideClosestPoint<W, B, Prim, PRECISE, true, STATS, 0><<<g, b, 0, s>>>(
                l.nodes, l.prims, l.spheres, l.perm, l.roots, l.out, l.sel, l.n, l.recordNormal, l.counter, l.errorWord,
                l.stats);
    } else {
        if (l.shortStack)
            kWideClosestPoint<W, B, Prim, PRECISE, false, STATS, kShortStack><<<g, b, 0, s>>>(
                l.nodes, l.prims, l.spheres, l.perm, l.roots, l.out, l.sel, l.n, l.recordNormal, l.counter, l.errorWord,
                l.stats);
        else
            kWideClosestPoint<W, B, Prim, PRECISE, false, STATS, 0><<<g, b, 0, s>>>(
                l.nodes, l.prims, l.spheres, l.perm, l.roots, l.out, l.sel, l.n, l.recordNormal, l.counter, l.errorWord,
                l.stats);
    }
    return cudaGetLastError();
}
// Precise mode on triangles: the traversal writes leaf positions to l.sel,
// then the refinement pass (launchRefineTriangles) writes the records.
template<int W, int B, class Prim>
cudaError_t launchWideClosestPrim(bool precise, const WideLaunch &l, cudaStream_t s) {
    if (precise) {
        if (Prim::kRefinePass && !l.sel) return cudaErrorInvalidValue;
        cudaError_t e = l.stats ? launchWideClosestKernel<W, B, Prim, true, true>(l, s)
                                : launchWideClosestKernel<W, B, Prim, true, false>(l, s);
        if (e != cudaSuccess || !Prim::kRefinePass || l.deferRefine) return e;
        return launchRefineTriangles(l.prims, l.spheres, l.perm, l.sel, l.out, l.n, l.recordNormal, s);
    }
    return l.stats ? launchWideClosestKernel<W, B, Prim, false, true>(l, s)
                   : launchWideClosestKernel<W, B, Prim, false, false>(l, s);
}
template<int W> cudaError_t launchWideClosestT(int bits, int dim, bool precise, const WideLaunch &l, cudaStream_t s) {
    if (dim == 3) {
        if (bits == 8) return launchWideClosestPrim<W, 8, Tri48Prim>(precise, l, s);
        if (bits == 16) return launchWideClosestPrim<W, 16, Tri48Prim>(precise, l, s);
        return launchWideClosestPrim<W, 32, Tri48Prim>(precise, l, s);
    }
    if (bits == 8) return launchWideClosestPrim<W, 8, Seg24Prim>(precise, l, s);
    if (bits == 16) return launchWideClosestPrim<W, 16, Seg24Prim>(precise, l, s);
    return launchWideClosestPrim<W, 32, Seg24Prim>(precise, l, s);
}
template<int W> cudaError_t launchRequantizeT(int bits, unsigned char *wideNodes, const int32_t *childBinary,
                                              const unsigned char *binNodes, int binStride, uint32_t nWide,
                                              uint32_t *errorWord, cudaStream_t s);

#define FCPWGB_WIDE_INSTANTIATE(W)                                                                                \
    template cudaError_t launchWideClosestT<W>(int bits, int dim, bool precise, const WideLaunch &l,              \
                                               cudaStream_t s);                                                   \
    template<> cudaError_t launchWideRayT<W>(int bits, int dim, const WideRayLaunch &l, cudaStream_t s) {         \
        if (l.n == 0) return cudaSuccess;                                                                          \
        dim3 g((l.n + 127) / 128), b(128);                                                                         \
        auto go = [&](auto kern) {                                                                                 \
            kern<<<g, b, 0, s>>>(l.nodes, l.prims, l.rays, l.perm, l.out, l.n, l.occl, l.callerRays, l.sortInfo,  \
                                 l.errorWord, l.stats);                                                            \
        };                                                                                                         \
        auto refill = [&](auto kern) {                                                                             \
            kern<<<dim3(l.grid), b, 0, s>>>(l.nodes, l.prims, l.rays, l.perm, l.out, l.n, l.occl, l.callerRays,     \
                                            l.sortInfo, l.counter, l.errorWord, l.stats);                          \
        };                                                                                                         \
        if (l.counter) {                                                                                           \
            if (dim == 3) {                                                                                        \
                if (bits == 8) refill(kWideRayRefill<W, 8, Tri48Prim>);                                            \
                else if (bits == 16) refill(kWideRayRefill<W, 16, Tri48Prim>);                                    \
                else refill(kWideRayRefill<W, 32, Tri48Prim>);                                                     \
            } else {                                                                                               \
                if (bits == 8) refill(kWideRayRefill<W, 8, Seg24Prim>);                                            \
                else if (bits == 16) refill(kWideRayRefill<W, 16, Seg24Prim>);                                    \
                else refill(kWideRayRefill<W, 32, Seg24Prim>);                                                     \
            }                                                                                                      \
        } else if (dim == 3) {                                                                                     \
            if (bits == 8) l.packet ? go(kWidePacketRay<W, 8, Tri48Prim>) : go(kWideRay<W, 8, Tri48Prim>);         \
            else if (bits == 16) l.packet ? go(kWidePacketRay<W, 16, Tri48Prim>) : go(kWideRay<W, 16, Tri48Prim>); \
            else l.packet ? go(kWidePacketRay<W, 32, Tri48Prim>) : go(kWideRay<W, 32, Tri48Prim>);                 \
        } else {                                                                                                   \
            if (bits == 8) l.packet ? go(kWidePacketRay<W, 8, Seg24Prim>) : go(kWideRay<W, 8, Seg24Prim>);         \
            else if (bits == 16) l.packet ? go(kWidePacketRay<W, 16, Seg24Prim>) : go(kWideRay<W, 16, Seg24Prim>); \
            else l.packet ? go(kWidePacketRay<W, 32, Seg24Prim>) : go(kWideRay<W, 32, Seg24Prim>);                 \
        }                                                                                                          \
        return cudaGetLastError();                                                                                 \
    }                                                                                                              \
    template<> cudaError_t launchRequantizeT<W>(int bits, unsigned char *wideNodes, const int32_t *childBinary,    \
                                                const unsigned char *binNodes, int binStride, uint32_t nWide,      \
                                                uint32_t *errorWord, cudaStream_t s) {                             \
        if (nWide == 0) return cudaSuccess;                                                                        \
        dim3 g((nWide + 127) / 128), b(128);                                                                       \
        if (bits == 8) kRequantize<W, 8><<<g, b, 0, s>>>(wideNodes, childBinary, binNodes, binStride, nWide, errorWord); \
        else if (bits == 16) kRequantize<W, 16><<<g, b, 0, s>>>(wideNodes, childBinary, binNodes, binStride, nWide, errorWord); \
        else kRequantize<W, 32><<<g, b, 0, s>>>(wideNodes, childBinary, binNodes, binStride, nWide, errorWord); \
        return cudaGetLastError();                                                                                 \
    }

}  // namespace fcpwgb
