// Closest silhouette points on the wide trees of an SNCH scene
// (Bvh.findClosestSilhouettePoint, bvh.slang:505-646, and its CPU twin
// bvh.inl:1435-1596, restated for W-wide nodes and warp packets).
//
// The wide tree is the collapse of the transferred binary SNCH tree with
// float child boxes and unmerged leaves, so every child slot is one binary
// node: its box is that node's box and kWideCones copies that node's normal
// cone and silhouette range into a per-slot record. A child is visited, as in
// the reference, when it has a cone (halfAngle >= 0), its box is within the
// query's current radius and the cone overlaps the view cone of its box
// (coneOverlap on the same box and squared distance). Leaves test their
// silhouette references with the reference's silhouette tests. The 32 queries
// of a warp walk the tree as one packet (kWidePacketClosestPoint's scheme).
//
// Equal distances: the reference keeps the later candidate of its visiting
// order; here the earlier silhouette reference wins, so the answer does not
// depend on the layout, the packet or the order of the queries. With a
// positive squared minimum radius the reference stops at the first
// silhouette found within it, which depends on its visiting order: that case
// stays on the binary kernel (k_binary.cu).
#include "k_wide.cuh"
#include "silhouette.cuh"

namespace fcpwgb {

namespace {

// per child slot: axis.xyz, halfAngle (< 0: no silhouettes below), radius,
// silhouette count and offset (leaf slots), padding
struct WideCone {
    float4 a;
    float4 b;
};
static_assert(sizeof(WideCone) == 32, "cone record");

__global__ void kWideCones(const int32_t *__restrict__ childBinary, const unsigned char *__restrict__ binNodes,
                           uint32_t nSlots, WideCone *__restrict__ cones) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nSlots) return;
    const int32_t b = childBinary[i];
    WideCone w;
    w.a = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    w.b = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (b >= 0) {
        const NodeCone c = loadCone(binNodes, (uint32_t)b);
        w.a = make_float4(c.axis.x, c.axis.y, c.axis.z, c.halfAngle);
        w.b = make_float4(c.radius, __uint_as_float(c.nSil), __uint_as_float(c.silOffset), 0.0f);
    }
    cones[i] = w;
}

template<int W, class Sil, int DIM>
__global__ void __launch_bounds__(kWideBlock, 8) kWidePacketSilhouette(const unsigned char *__restrict__ nodes,
                                                                    const WideCone *__restrict__ cones,
                                                                    const unsigned char *__restrict__ sils,
                                                                    const DevSphere *__restrict__ spheres,
                                                                    const uint32_t *__restrict__ flip,
                                                                    const uint32_t *__restrict__ perm,
                                                                    DevInteraction *__restrict__ out, uint32_t n,
                                                                    float sqMinR, float precision,
                                                                    uint32_t *errorWord) {
    constexpr uint32_t kSlotMask = W - 1;
    constexpr int kWarps = kWideBlock / 32;
    __shared__ uint32_t sRef[kWarps][kPacketShort];
    __shared__ float sDist[kWarps][kPacketShort][32];
    uint32_t lRef[kWideStack - kPacketShort];
    float lDist[kWideStack - kPacketShort];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t i = blockIdx.x * kWideBlock + threadIdx.x;
    const bool valid = i < n;
    const uint32_t slot = valid ? (perm ? __ldg(perm + i) : i) : 0u;  // the caller's slot
    float3 c = make_float3(0.f, 0.f, 0.f);
    float r2 = -1.0f;
    bool flipNormal = false;
    if (valid) {
        const float4 s4 = ldg4(spheres + i);
        c = make_float3(s4.x, s4.y, s4.z);
        r2 = s4.w;
        flipNormal = __ldg(flip + slot) != 0;
    }
    DevInteraction best = defaultInteraction();
    uint32_t bestPos = kUintMax;
    WideNodeRegs<W, 32> node;

    bool act = valid && !(sqMinR >= r2);  // this lane needs the current record
    uint32_t cur = 0;
    int sp = 0;  // warp-uniform
    if (__ballot_sync(0xffffffffu, act)) {
        for (;;) {
            bool descend = false;
            if (!(cur & kLeafBit)) {
                node.load(nodes, cur);
                float d2[W];
                bool need[W];
#pragma unroll
                for (int k = 0; k < W; k++) {
                    const WideCone wc = cones[(size_t)cur * W + k];
                    const float3 lo = make_float3(node.bound(0, k), node.bound(1, k), node.bound(2, k));
                    const float3 hi = make_float3(node.bound(3, k), node.bound(4, k), node.bound(5, k));
                    d2[k] = boxSphereD2Min(lo, hi, c);
                    need[k] = act && node.cnt(k) != kWideEmpty && wc.a.w >= 0.0f && d2[k] <= r2;
                    if (need[k])
                        need[k] = coneOverlap<DIM>(make_float3(wc.a.x, wc.a.y, wc.a.z), wc.a.w, wc.b.x, c, lo, hi,
                                                   d2[k]);
                }
                // children needed by any lane, ordered by the first active lane's distances
                const uint32_t leader = __ffs(__ballot_sync(0xffffffffu, act)) - 1;
                uint32_t key[W];
                int nh = 0;
#pragma unroll
                for (int k = 0; k < W; k++) {
                    const bool any = __ballot_sync(0xffffffffu, need[k]) != 0;
                    const float lead = __shfl_sync(0xffffffffu, need[k] ? d2[k] : kFltMax, leader);
                    key[k] = any ? ((__float_as_uint(lead) & ~kSlotMask) | (uint32_t)k) : 0xffffffffu;
                    nh += any ? 1 : 0;
                }
                sortNetwork<W>(key);
                if (nh > 0) {
                    if (sp + nh - 1 > kWideStack) {
                        if (lane == 0) atomicOr(errorWord, kErrStackOverflow);
                        break;
                    }
                    uint32_t refs[W];
                    float mine[W];
#pragma unroll
                    for (int k = 0; k < W; k++) {
                        refs[k] = node.cnt(k) == 0 ? node.ref(k) : (kLeafBit | (cur * W + (uint32_t)k));
                        mine[k] = need[k] ? d2[k] : __int_as_float(0x7fc00000);  // NaN: never <= r2
                    }
#pragma unroll
                    for (int k = W - 1; k >= 0; k--) {
                        if (k < nh) {
                            const uint32_t s = key[k] & kSlotMask;
                            const uint32_t packed = selectBySlot<W>(refs, s);
                            const float dl = selectBySlot<W>(mine, s);
                            if (k == 0) {
                                cur = packed;
                                act = dl <= r2;
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
                const WideCone wc = cones[cur & ~kLeafBit];
                const uint32_t nSil = __float_as_uint(wc.b.y), off = __float_as_uint(wc.b.z);
                for (uint32_t p = 0; p < nSil; p++) {
                    const Sil sil = Sil::load(sils, off + p);
                    if (act && sil.index != best.index) {
                        DevInteraction cI = defaultInteraction();
                        if (sil.closestSilhouettePoint(c, r2, flipNormal, sqMinR, precision, cI) &&
                            (bestPos == kUintMax || cI.d < best.d || (cI.d == best.d && off + p < bestPos))) {
                            r2 = fminf(r2, cI.d * cI.d);
                            best = cI;
                            bestPos = off + p;
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
                act = dl <= r2 && !(sqMinR >= r2);
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
}

template<int W>
cudaError_t launchSilW(int dim, const WideSilLaunch &l, cudaStream_t s) {
    const dim3 g((l.n + kWideBlock - 1) / kWideBlock), b(kWideBlock);
    const WideCone *cones = (const WideCone *)l.cones;
    if (dim == 3)
        kWidePacketSilhouette<W, EdgeSil, 3><<<g, b, 0, s>>>(l.nodes, cones, l.sils, l.spheres, l.flip, l.perm, l.out,
                                                             l.n, l.sqMinR, l.precision, l.errorWord);
    else
        kWidePacketSilhouette<W, VertexSil, 2><<<g, b, 0, s>>>(l.nodes, cones, l.sils, l.spheres, l.flip, l.perm,
                                                               l.out, l.n, l.sqMinR, l.precision, l.errorWord);
    return cudaGetLastError();
}

}  // namespace

size_t wideConeBytes() { return sizeof(WideCone); }

cudaError_t launchWideCones(const int32_t *childBinary, const unsigned char *binNodes, uint32_t nSlots, void *cones,
                            cudaStream_t s) {
    if (nSlots == 0) return cudaSuccess;
    kWideCones<<<(nSlots + 255) / 256, 256, 0, s>>>(childBinary, binNodes, nSlots, (WideCone *)cones);
    return cudaGetLastError();
}

cudaError_t launchWideSilhouette(int W, int dim, const WideSilLaunch &l, cudaStream_t s) {
    if (l.n == 0) return cudaSuccess;
    switch (W) {
        case 2: return launchSilW<2>(dim, l, s);
        case 4: return launchSilW<4>(dim, l, s);
        default: return launchSilW<8>(dim, l, s);
    }
}

}  // namespace fcpwgb
