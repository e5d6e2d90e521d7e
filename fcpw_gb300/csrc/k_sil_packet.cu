// Closest silhouette points with warp packets on the binary SNCH tree
// (Bvh.findClosestSilhouettePoint, bvh.slang:505-646, and its CPU twin
// bvh.inl:1435-1596). The 32 (spatially sorted) queries of a warp walk the
// tree together: every node record is loaded once for the warp, and each
// lane applies the reference's tests to its own query -- a child is visited
// when it has a normal cone (halfAngle >= 0), its box is within the query's
// radius and the cone overlaps the view cone of its box (coneOverlapFast,
// which decides as coneOverlap, on the same box and squared distance) -- and
// a lane takes part in a subtree only
// while it passes them. The children go in the order of the first active
// lane's distances, the farther one onto a warp stack (shared memory, one
// distance column per lane) that is re-checked against each lane's radius
// when popped.
//
// Equal distances: the reference keeps the later candidate of its own
// visiting order. Here boxes are visited within the winner's distance plus
// the rounding band of the closest-point kernels (bandRadius2), so every
// candidate at the winner's distance is tested, and the earliest silhouette
// reference wins (over all listings of the tied silhouettes): the answer
// does not depend on which queries share a warp or on their order. (A wide
// collapse of the tree would skip the cone tests of the collapsed binary
// nodes, whose outcome is not monotone in floating point, so the packets
// walk the binary nodes.) With a positive squared minimum radius the
// reference stops at the first silhouette found within it, which depends on
// its visiting order: that case stays on the binary kernel (k_binary.cu). A
// query whose centre is not finite gets the default record.
#include "k_wide.cuh"
#include "silhouette.cuh"

namespace fcpwgb {

namespace {

constexpr int kSilShort = 32;  // warp-stack entries in shared memory; deeper ones in registers/local

// With `counter` non-NULL the blocks are persistent (one resident wave) and
// every warp takes its next packet of 32 sorted queries from the counter as
// soon as its previous one is done. With STATS, per-launch totals go to
// stats[0..4]: warp steps at an inner node (two 64 B child records loaded),
// warp steps at a leaf, silhouette records loaded by warps, and the lanes'
// child tests and silhouette tests.
template<class Sil, int DIM, bool STATS>
__global__ void __launch_bounds__(kWideBlock, 8) kPacketSilhouette(const unsigned char *__restrict__ nodes,
                                                                const unsigned char *__restrict__ sils,
                                                                const DevSphere *__restrict__ spheres,
                                                                const uint32_t *__restrict__ flip,
                                                                const uint32_t *__restrict__ perm,
                                                                DevInteraction *__restrict__ out, uint32_t n,
                                                                float sqMinR, float precision, uint32_t *counter,
                                                                uint32_t *errorWord, unsigned long long *stats) {
    Count<STATS> wInner, wLeaf, wSil, tChild, tSil;
    constexpr int kWarps = kWideBlock / 32;
    __shared__ uint32_t sRef[kWarps][kSilShort];
    __shared__ float sDist[kWarps][kSilShort][32];
    uint32_t lRef[kStackDepth - kSilShort];
    float lDist[kStackDepth - kSilShort];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
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
        const uint32_t slot = valid ? (perm ? __ldg(perm + i) : i) : 0u;  // the caller's slot
        float3 c = make_float3(0.f, 0.f, 0.f);
        float r2 = -1.0f;
        bool flipNormal = false;
        if (valid) {
            const float4 s4 = ldg4(spheres + i);
            c = make_float3(s4.x, s4.y, s4.z);
            r2 = queryRadius2(c, s4.w);
            flipNormal = __ldg(flip + slot) != 0;
        }
        DevInteraction best = defaultInteraction();
        uint32_t bestPos = kUintMax;
        // boxes are pruned against rp2: the radius widened by the rounding band
        float rp2 = bandRadius2(sqrtf(r2), c);

        const NodeBox root = loadNode<64>(nodes, 0);
        bool act = valid && !(sqMinR >= r2) && boxSphereD2Min(root.pMin, root.pMax, c) <= rp2;
        uint32_t cur = 0;
        int sp = 0;  // warp-uniform
        if (__ballot_sync(0xffffffffu, act)) {
            for (;;) {
                const NodeBox node = loadNode<64>(nodes, cur);
                bool next = false;
                if (node.nPrims > 0) {
                    const NodeCone cone = loadCone(nodes, cur);
                    wLeaf.add(1);
                    wSil.add(cone.nSil);
                    if (act) tSil.add(cone.nSil);
                    for (uint32_t p = 0; p < cone.nSil; p++) {
                        const Sil sil = Sil::load(sils, cone.silOffset + p);
                        const uint32_t pos = cone.silOffset + p;
                        if (act && sil.index == best.index) {
                            // the winner again, listed in another leaf (an edge is listed for both of
                            // its faces): not tested again, as in the reference, but its earliest
                            // listing is what a tie compares against
                            bestPos = min(bestPos, pos);
                        } else if (act) {
                            DevInteraction cI = defaultInteraction();
                            if (sil.closestSilhouettePoint(c, r2, flipNormal, sqMinR, precision, cI) &&
                                (bestPos == kUintMax || cI.d < best.d || (cI.d == best.d && pos < bestPos))) {
                                r2 = fminf(r2, cI.d * cI.d);
                                rp2 = bandRadius2(cI.d, c);
                                best = cI;
                                bestPos = pos;
                            }
                        }
                    }
                } else {
                    const uint32_t li = cur + 1, ri = cur + node.offset;
                    wInner.add(1);
                    if (act) tChild.add(2);
                    const NodeCone lc = loadCone(nodes, li), rc = loadCone(nodes, ri);
                    const NodeBox lb = loadNode<64>(nodes, li), rb = loadNode<64>(nodes, ri);
                    float dl = 0.0f, dr = 0.0f;
                    bool hitL = act && lc.halfAngle >= 0.0f, hitR = act && rc.halfAngle >= 0.0f;
                    if (hitL) {
                        dl = boxSphereD2Min(lb.pMin, lb.pMax, c);
                        hitL = dl <= rp2 && coneOverlapFast<DIM>(lc.axis, lc.halfAngle, lc.radius, c, lb.pMin, lb.pMax, dl);
                    }
                    if (hitR) {
                        dr = boxSphereD2Min(rb.pMin, rb.pMax, c);
                        hitR = dr <= rp2 && coneOverlapFast<DIM>(rc.axis, rc.halfAngle, rc.radius, c, rb.pMin, rb.pMax, dr);
                    }
                    const bool anyL = __ballot_sync(0xffffffffu, hitL) != 0, anyR = __ballot_sync(0xffffffffu, hitR) != 0;
                    if (anyL || anyR) {
                        bool takeR = !anyL;
                        if (anyL && anyR) {
                            // the first active lane's nearer child first (the reference's order for that lane)
                            const uint32_t leader = __ffs(__ballot_sync(0xffffffffu, act)) - 1;
                            const float ldl = __shfl_sync(0xffffffffu, hitL ? dl : kFltMax, leader);
                            const float ldr = __shfl_sync(0xffffffffu, hitR ? dr : kFltMax, leader);
                            takeR = ldr < ldl;
                            if (sp >= kStackDepth) {
                                if (lane == 0) atomicOr(errorWord, kErrStackOverflow);
                                break;
                            }
                            const uint32_t other = takeR ? li : ri;
                            const float dOther = (takeR ? hitL : hitR) ? (takeR ? dl : dr) : __int_as_float(0x7fc00000);
                            if (sp < kSilShort) {
                                if (lane == 0) sRef[warp][sp] = other;
                                sDist[warp][sp][lane] = dOther;  // NaN: this lane does not need it
                            } else {
                                lRef[sp - kSilShort] = other;
                                lDist[sp - kSilShort] = dOther;
                            }
                            sp++;
                            __syncwarp();
                        }
                        cur = takeR ? ri : li;
                        act = takeR ? hitR : hitL;
                        next = true;
                    }
                }
                if (next) continue;
                // pop until some lane needs the entry
                while (sp > 0) {
                    sp--;
                    uint32_t ref;
                    float d;
                    if (sp < kSilShort) {
                        ref = sRef[warp][sp];
                        d = sDist[warp][sp][lane];
                    } else {
                        ref = lRef[sp - kSilShort];
                        d = lDist[sp - kSilShort];
                    }
                    act = d <= rp2 && !(sqMinR >= r2);
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
        if (valid) out[slot] = best;
        if (!counter) break;
    }
    if (STATS && stats) {
        const uint32_t lane = threadIdx.x & 31u;
        if (lane == 0) {
            atomicAdd(stats + 0, wInner.get());
            atomicAdd(stats + 1, wLeaf.get());
            atomicAdd(stats + 2, wSil.get());
        }
        atomicAdd(stats + 3, tChild.get());
        atomicAdd(stats + 4, tSil.get());
    }
}

}  // namespace

cudaError_t launchSilhouettePacket(const SceneView &v, const DevSphere *spheres, const uint32_t *flip,
                                   const uint32_t *perm, DevInteraction *out, uint32_t n, float sqMinR,
                                   float precision, uint32_t *counter, uint32_t grid, cudaStream_t s,
                                   unsigned long long *stats) {
    if (n == 0) return cudaSuccess;
    const dim3 g(counter ? grid : (n + kWideBlock - 1) / kWideBlock), b(kWideBlock);
    if (v.dim == 3) {
        if (stats)
            kPacketSilhouette<EdgeSil, 3, true><<<g, b, 0, s>>>(v.nodes, v.sils, spheres, flip, perm, out, n, sqMinR,
                                                                precision, counter, v.errorWord, stats);
        else
            kPacketSilhouette<EdgeSil, 3, false><<<g, b, 0, s>>>(v.nodes, v.sils, spheres, flip, perm, out, n, sqMinR,
                                                                 precision, counter, v.errorWord, nullptr);
    } else {
        if (stats)
            kPacketSilhouette<VertexSil, 2, true><<<g, b, 0, s>>>(v.nodes, v.sils, spheres, flip, perm, out, n, sqMinR,
                                                                  precision, counter, v.errorWord, stats);
        else
            kPacketSilhouette<VertexSil, 2, false><<<g, b, 0, s>>>(v.nodes, v.sils, spheres, flip, perm, out, n,
                                                                   sqMinR, precision, counter, v.errorWord, nullptr);
    }
    return cudaGetLastError();
}

}  // namespace fcpwgb
