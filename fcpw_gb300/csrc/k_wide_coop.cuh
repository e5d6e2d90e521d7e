// Cooperative schedule of the wide closest-point traversal: a group of L = 2,
// 4 or 8 consecutive lanes answers one (sorted) query. Included by k_wide.cuh
// after the helpers it uses.
//
// Per inner record, lane j of the group loads and tests only its own child
// slots (j, j + L, ...): their counts, references and the six bounds straight
// from the record (the group's lanes read the same cache lines), the box
// distances and, before the query's first primitive, the far distances, whose
// minimum over the group shrinks the radius. The group then gathers the W
// child keys (distance bits, slot in the low bits) into every lane, sorts them
// with the same network as the one-thread schedule, continues with the
// nearest child needed and pushes the others, farthest first, onto the
// group's stack (entries in shared memory, one writer per entry; deeper
// entries in every lane's local memory). Per leaf, lane j tests primitives
// j, j + L, ... of the leaf, and the group reduces their candidates with the
// rules of beatsWinner: the winner is the least (distance, leaf position)
// among the qualifying candidates (every candidate once a primitive has been
// found, else those within the radius), and in precise mode the runner-up is
// the least candidate other than the winner over everything tested, kept from
// the two least candidates of each leaf. The group's state (radius, winner,
// runner-up, stack pointer, current record) is identical in its lanes, so
// every shuffle is over the whole group and the group's control flow stays
// uniform; the answers equal those of the other schedules byte for byte.
#pragma once

namespace fcpwgb {

constexpr int kCoopShort = 32;  // group stack entries kept in shared memory

template<int L> struct LaneGroup {
    uint32_t mask;  // the group's lanes in the warp
    uint32_t j;     // lane within the group
    FCPWGB_D LaneGroup() {
        const uint32_t lane = threadIdx.x & 31u;
        j = lane & (uint32_t)(L - 1);
        mask = ((1u << L) - 1u) << (lane & ~(uint32_t)(L - 1));
    }
    template<class T> FCPWGB_D T from(T v, uint32_t src) const { return __shfl_sync(mask, v, (int)src, L); }
    template<class T> FCPWGB_D T xorShfl(T v, int o) const { return __shfl_xor_sync(mask, v, o, L); }
    FCPWGB_D float minAll(float v) const {
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) v = fminf(v, xorShfl(v, o));
        return v;
    }
};

// (distance, leaf position) candidates in the order of beatsWinner; an absent
// candidate is (+inf, kUintMax), a NaN distance is never taken
struct Cand {
    float d;
    uint32_t s;
};
FCPWGB_D Cand noCand() { return Cand{__int_as_float(0x7f800000), kUintMax}; }
FCPWGB_D bool candLess(Cand a, Cand b) { return a.d < b.d || (a.d == b.d && a.s < b.s); }
FCPWGB_D Cand candMin(Cand a, Cand b) { return candLess(b, a) ? b : a; }
FCPWGB_D Cand candMax(Cand a, Cand b) { return candLess(b, a) ? a : b; }
template<int L> FCPWGB_D Cand groupMin(const LaneGroup<L> &g, Cand a) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
        Cand b{g.xorShfl(a.d, o), g.xorShfl(a.s, o)};
        a = candMin(a, b);
    }
    return a;
}
// the two least candidates of the group (a1 <= a2 in every lane on entry)
template<int L> FCPWGB_D void groupTop2(const LaneGroup<L> &g, Cand &a1, Cand &a2) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
        Cand b1{g.xorShfl(a1.d, o), g.xorShfl(a1.s, o)};
        Cand b2{g.xorShfl(a2.d, o), g.xorShfl(a2.s, o)};
        Cand lo = candMin(a1, b1), mid = candMin(candMax(a1, b1), candMin(a2, b2));
        a1 = lo;
        a2 = mid;
    }
}

// one child slot of wide record `rec`, read from memory: its count byte, its
// reference and its box's squared min (and, with far, max) distance to c, on
// the dequantised bounds fmaf(q, 2^e, origin) the quantiser checked
template<int W, int BITS> struct SlotBox {
    using Lay = WideLayout<W, BITS>;
    FCPWGB_D static float bound(const unsigned char *rec, const uint4 &hdr, int k, uint32_t slot) {
        const uint32_t idx = (uint32_t)k * W + slot;
        if constexpr (BITS == 32) {
            return __ldg(reinterpret_cast<const float *>(rec + Lay::kBounds) + idx);
        } else {
            const int a = k % 3;
            const float q = BITS == 16 ? (float)__ldg(reinterpret_cast<const unsigned short *>(rec + Lay::kBounds) + idx)
                                       : (float)__ldg(rec + Lay::kBounds + idx);
            const float o = __uint_as_float(a == 0 ? hdr.x : (a == 1 ? hdr.y : hdr.z));
            const float s = exp2i((int)((hdr.w >> (8 * a)) & 0xffu) - 127);
            return __fmaf_rn(q, s, o);
        }
    }
    FCPWGB_D static float d2Min(const unsigned char *rec, const uint4 &hdr, uint32_t slot, float3 c, float &d2Max,
                                bool far) {
        const float lx = bound(rec, hdr, 0, slot), ly = bound(rec, hdr, 1, slot), lz = bound(rec, hdr, 2, slot);
        const float hx = bound(rec, hdr, 3, slot), hy = bound(rec, hdr, 4, slot), hz = bound(rec, hdr, 5, slot);
        const float ax = fmax3(lx - c.x, c.x - hx, 0.0f);
        const float ay = fmax3(ly - c.y, c.y - hy, 0.0f);
        const float az = fmax3(lz - c.z, c.z - hz, 0.0f);
        if (far) {
            float lo, hi;
            boxSphereDist(make_float3(lx, ly, lz), make_float3(hx, hy, hz), c, lo, hi);
            d2Max = hi;
        }
        return ax * ax + ay * ay + az * az;
    }
};

template<int W, int BITS, class Prim, bool PRECISE, bool STATS, int L>
__global__ void __launch_bounds__(kWideBlock, 8) kWideCoopClosestPoint(const unsigned char *__restrict__ nodes,
                                                                    const unsigned char *__restrict__ prims,
                                                                    const DevSphere *__restrict__ spheres,
                                                                    const uint32_t *__restrict__ perm,
                                                                    const uint32_t *__restrict__ roots,
                                                                    DevInteraction *__restrict__ out,
                                                                    uint2 *__restrict__ sel, uint32_t n,
                                                                    int recordNormal, uint32_t *errorWord,
                                                                    unsigned long long *stats) {
    using Lay = WideLayout<W, BITS>;
    constexpr uint32_t kSlotMask = W - 1;
    constexpr int kGroups = kWideBlock / L;
    constexpr int kMine = (W + L - 1) / L;  // child slots per lane
    __shared__ uint32_t sRef[kGroups][kCoopShort];
    __shared__ float sDist[kGroups][kCoopShort];
    uint32_t lRef[kWideStack - kCoopShort];  // deeper entries, the same in every lane of the group
    float lDist[kWideStack - kCoopShort];
    const LaneGroup<L> grp;
    const uint32_t gi = threadIdx.x / L;
    const uint32_t i = blockIdx.x * kGroups + gi;
    if (i >= n) return;  // the whole group leaves together
    const float4 s4 = ldg4(spheres + i);
    const float3 c = make_float3(s4.x, s4.y, s4.z);
    const float r2User = queryRadius2(c, s4.w);
    float r2 = r2User;
    DevInteraction best = defaultInteraction();
    uint32_t selected = kUintMax;
    bool found = false;
    NearTie<PRECISE> tie;
    float rp2 = tie.prune(r2, c);
    Count<STATS> tExp, tTests;
    uint32_t cur = roots ? __ldg(roots + i) : 0u;
    int sp = 0;
    for (;;) {
        if (!(cur & kLeafBit)) {
            const unsigned char *rec = nodes + (size_t)cur * Lay::kSize;
            uint4 hdr = make_uint4(0u, 0u, 0u, 0u);
            if constexpr (BITS != 32) hdr = __ldg(reinterpret_cast<const uint4 *>(rec));
            if (grp.j == 0) tExp.add(1);
            float d2m[kMine];
            bool live[kMine];
            float far = kFltMax;
#pragma unroll
            for (int t = 0; t < kMine; t++) {
                const uint32_t slot = grp.j + (uint32_t)(t * L);
                live[t] = false;
                d2m[t] = kFltMax;
                if (slot < (uint32_t)W && __ldg(rec + Lay::kCnt + slot) != kWideEmpty) {
                    float d2Max = kFltMax;
                    d2m[t] = SlotBox<W, BITS>::d2Min(rec, hdr, slot, c, d2Max, !found);
                    live[t] = true;
                    far = fminf(far, d2Max);
                }
            }
            if (!found) {
                r2 = fminf(r2, grp.minAll(far));
                rp2 = tie.prune(r2, c);
            }
            uint32_t mine[kMine];
#pragma unroll
            for (int t = 0; t < kMine; t++) {
                const uint32_t slot = grp.j + (uint32_t)(t * L);
                mine[t] = live[t] && d2m[t] <= rp2 ? ((__float_as_uint(d2m[t]) & ~kSlotMask) | slot) : 0xffffffffu;
            }
            uint32_t key[W];
            int nh = 0;
#pragma unroll
            for (int s = 0; s < W; s++) {
                key[s] = grp.from(mine[s / L], (uint32_t)(s % L));
                nh += key[s] != 0xffffffffu ? 1 : 0;
            }
            sortNetwork<W>(key);
            if (nh > 0) {
                if (sp + nh - 1 > kWideStack) {
                    if (grp.j == 0) atomicOr(errorWord, kErrStackOverflow);
                    break;
                }
                const uint32_t *refs = reinterpret_cast<const uint32_t *>(rec + Lay::kRefs);
#pragma unroll
                for (int k = W - 1; k >= 1; k--) {
                    if (k < nh) {
                        const int at = sp + (nh - 1 - k);
                        const uint32_t slot = key[k] & kSlotMask;
                        const bool writer = grp.j == (uint32_t)(k % L);
                        if (at < kCoopShort) {
                            if (writer) {
                                const uint32_t cnt = __ldg(rec + Lay::kCnt + slot), ref = __ldg(refs + slot);
                                sRef[gi][at] = cnt == 0 ? ref : packLeaf(ref, cnt);
                                sDist[gi][at] = __uint_as_float(key[k] & ~kSlotMask);
                            }
                        } else {
                            const uint32_t cnt = __ldg(rec + Lay::kCnt + slot), ref = __ldg(refs + slot);
                            lRef[at - kCoopShort] = cnt == 0 ? ref : packLeaf(ref, cnt);
                            lDist[at - kCoopShort] = __uint_as_float(key[k] & ~kSlotMask);
                        }
                    }
                }
                sp += nh - 1;
                const uint32_t slot = key[0] & kSlotMask;
                const uint32_t cnt = __ldg(rec + Lay::kCnt + slot), ref = __ldg(refs + slot);
                cur = cnt == 0 ? ref : packLeaf(ref, cnt);
                __syncwarp(grp.mask);
                continue;
            }
        } else {
            const uint32_t off = cur & 0x07ffffffu, cnt = (cur >> 27) & 0xfu;
            if (grp.j == 0) tTests.add(cnt);
            Cand mq = noCand(), t1 = noCand(), t2 = noCand();
            float3 mp = make_float3(0.f, 0.f, 0.f);
            float2 muv = make_float2(0.f, 0.f);
            uint32_t mIndex = kUintMax;
            for (uint32_t p = grp.j; p < cnt; p += L) {
                const Prim prim = Prim::load(prims, off + p);
                float3 pt;
                float2 uv;
                const float d = prim.closestPoint(c, pt, uv);
                const Cand cd{d, off + p};
                if ((found || d * d <= r2) && candLess(cd, mq)) {
                    mq = cd;
                    mp = pt;
                    muv = uv;
                    mIndex = prim.index;
                }
                if (PRECISE) {
                    if (candLess(cd, t1)) {
                        t2 = t1;
                        t1 = cd;
                    } else if (candLess(cd, t2)) {
                        t2 = cd;
                    }
                }
            }
            const Cand w = groupMin<L>(grp, mq);
            if (PRECISE) groupTop2<L>(grp, t1, t2);
            const Cand old{best.d, selected};
            const bool wins = w.s != kUintMax && (!found || candLess(w, old));
            if (wins) {
                const uint32_t owner = (w.s - off) % (uint32_t)L;
                best.p = make_float3(grp.from(mp.x, owner), grp.from(mp.y, owner), grp.from(mp.z, owner));
                best.uv = make_float2(grp.from(muv.x, owner), grp.from(muv.y, owner));
                best.index = grp.from(mIndex, owner);
                best.n = make_float3(0.f, 0.f, 0.f);
                best.d = w.d;
            }
            if constexpr (PRECISE) {
                // runner-up: the least of the previous runner-up, the previous winner and the
                // leaf's two least candidates, other than the winner
                const uint32_t winSel = wins ? w.s : selected;
                Cand ru{tie.d2nd, tie.sel2nd};
                if (ru.s == winSel) ru = noCand();
                if (wins && found) ru = candMin(ru, old);
                if (t1.s != winSel) ru = candMin(ru, t1);
                if (t2.s != winSel) ru = candMin(ru, t2);
                if (ru.s != kUintMax) {
                    tie.d2nd = ru.d;
                    tie.sel2nd = ru.s;
                }
            }
            if (wins) {
                selected = w.s;
                found = true;
                r2 = fminf(r2, w.d * w.d);
                rp2 = tie.pruneHit(w.d, c);
            }
        }
        bool next = false;
        while (sp > 0) {
            sp--;
            const float dl = sp < kCoopShort ? sDist[gi][sp] : lDist[sp - kCoopShort];
            if (dl <= rp2) {
                cur = sp < kCoopShort ? sRef[gi][sp] : lRef[sp - kCoopShort];
                next = true;
                break;
            }
        }
        __syncwarp(grp.mask);
        if (!next) break;
    }
    if (grp.j == 0)
        finishQuery<Prim, PRECISE>(prims, perm, out, sel, i, c, r2User, found, selected, recordNormal, best, tie);
    if (STATS && stats && grp.j == 0) {
        atomicAdd(stats + 1, tExp.get());
        atomicAdd(stats + 2, tTests.get());
    }
}

}  // namespace fcpwgb
