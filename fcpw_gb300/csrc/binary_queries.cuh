// Per-query traversals of the transferred binary trees in the reference GPU
// order, as device functions: the kernels of k_binary.cu run them on a scene's
// tree, and the instanced kernels (instanced.cu) on each object's tree in
// object space.
#pragma once

#include "device_common.cuh"
#include "silhouette.cuh"

namespace fcpwgb {

// Bvh.intersect(sphere, randNums) with constant branch weights, bvh.slang:257-392
// (CPU twin bvh.inl:1140-1288): one stochastic descent chooses a child with
// probability proportional to its overlap weight, rescaling u = rn.x at every
// choice; in the leaf a primitive within the sphere is chosen in proportion to
// its surface area (every primitive counts when the leaf's box lies wholly
// inside the sphere), and a point is sampled on it with rn.y (, rn.z). `best`
// receives the sample (d = selection pdf x sample pdf) or the default record;
// returns whether a primitive was selected.
template<class Prim, int NODE_STRIDE>
FCPWGB_D bool sphereSampleBinary(const unsigned char *__restrict__ nodes, const unsigned char *__restrict__ prims,
                                 float3 c, float r2, float3 rn, uint32_t depthLimit, uint32_t *errorWord,
                                 DevInteraction &best) {
    best = defaultInteraction();
    uint32_t selected = kUintMax;
    bool didIntersect = false;
    NodeBox root = loadNode<NODE_STRIDE>(nodes, 0);
    float d2Min, d2Max;
    boxSphereDist(root.pMin, root.pMax, c, d2Min, d2Max);
    if (d2Min <= r2) {
        float maxDistToChild = d2Max;
        float traversalPdf = 1.0f;
        float u = rn.x;
        uint32_t ni = 0;
        for (uint32_t step = 0; step <= depthLimit; step++) {
            NodeBox node = loadNode<NODE_STRIDE>(nodes, ni);
            if (node.nPrims > 0) {
                float total = 0.0f;
                for (uint32_t p = 0; p < node.nPrims; p++) {
                    uint32_t pi = node.offset + p;
                    Prim prim = Prim::load(prims, pi);
                    DevInteraction cI = defaultInteraction();
                    bool hit = false;
                    if (maxDistToChild <= r2) {
                        hit = true;
                        cI.d = prim.surfaceArea();
                        cI.index = prim.index;
                    } else {
                        float3 pt;
                        float2 uv;
                        float d = prim.closestPoint(c, pt, uv);
                        if (d * d <= r2) {
                            hit = true;
                            cI.p = pt;
                            cI.uv = uv;
                            cI.d = prim.surfaceArea();
                            cI.index = prim.index;
                        }
                    }
                    if (hit) {
                        didIntersect = true;
                        total += cI.d;
                        float prob = cI.d / total;
                        if (u < prob) {
                            u = u / prob;
                            best = cI;
                            best.d *= traversalPdf;
                            selected = pi;
                        } else {
                            u = (u - prob) / (1.0f - prob);
                        }
                    }
                }
                if (total > 0.0f) best.d /= total;
                break;
            }
            uint32_t li = ni + 1, ri = ni + node.offset;
            NodeBox l = loadNode<NODE_STRIDE>(nodes, li);
            NodeBox r = loadNode<NODE_STRIDE>(nodes, ri);
            float l0, l1, r0, r1;
            boxSphereDist(l.pMin, l.pMax, c, l0, l1);
            boxSphereDist(r.pMin, r.pMax, c, r0, r1);
            float wl = l0 <= r2 ? 1.0f : 0.0f;
            float wr = r0 <= r2 ? 1.0f : 0.0f;
            float total = wl + wr;
            if (!(total > 0.0f)) break;
            float pl = wl / total, pr = 1.0f - pl;
            if (u < pl) {
                u = u / pl;
                ni = li;
                traversalPdf *= pl;
                maxDistToChild = l1;
            } else {
                u = (u - pl) / pr;
                ni = ri;
                traversalPdf *= pr;
                maxDistToChild = r1;
            }
            if (step == depthLimit) atomicOr(errorWord, kErrStepBudget);
        }
    }
    if (didIntersect) {
        if (best.index == kUintMax || selected == kUintMax) {
            didIntersect = false;
        } else {
            Prim prim = Prim::load(prims, selected);
            float pdf = prim.samplePoint(make_float2(rn.y, rn.z), best.uv, best.p, best.n);
            best.d *= pdf;
        }
    }
    if (!didIntersect) best = defaultInteraction();
    return didIntersect;
}

// Bvh.findClosestSilhouettePoint, bvh.slang:505-646 (CPU twin bvh.inl:1435-1596),
// on a binary SNCH tree (64 B node records): depth first, nearer child first,
// a child entered when its cone is valid, its box within the radius and the
// view cone of its box overlaps its normal cone; r2 shrinks to every
// silhouette point found, and the search stops once it is within the minimum
// radius. `best` receives the closest silhouette point (or the default
// record); r2 returns the final squared radius. Returns whether one was found.
template<class Sil, int DIM>
FCPWGB_D bool silhouetteBinary(const unsigned char *__restrict__ nodes, const unsigned char *__restrict__ sils,
                               float3 c, float &r2, bool flipNormal, float sqMinR, float precision,
                               uint32_t *errorWord, DevInteraction &best) {
    best = defaultInteraction();
    bool found = false;
    if (sqMinR >= r2) return false;
    uint32_t stack[kStackDepth];
    NodeBox root = loadNode<64>(nodes, 0);
    if (!(boxSphereD2Min(root.pMin, root.pMax, c) <= r2)) return false;
    stack[0] = 0;
    int sp = 0;
    while (sp >= 0) {
        uint32_t ni = stack[sp--];
        NodeBox node = loadNode<64>(nodes, ni);
        if (!(boxSphereD2Min(node.pMin, node.pMax, c) <= r2)) continue;
        if (node.nPrims > 0) {
            NodeCone cone = loadCone(nodes, ni);
            for (uint32_t p = 0; p < cone.nSil; p++) {
                Sil sil = Sil::load(sils, cone.silOffset + p);
                if (sil.index == best.index) continue;  // already checked
                DevInteraction cI = defaultInteraction();
                if (sil.closestSilhouettePoint(c, r2, flipNormal, sqMinR, precision, cI)) {
                    r2 = fminf(r2, cI.d * cI.d);
                    best = cI;
                    found = true;
                    if (sqMinR >= r2) break;
                }
            }
        } else {
            uint32_t li = ni + 1, ri = ni + node.offset;
            float dl = 0.0f, dr = 0.0f;
            NodeCone lc = loadCone(nodes, li);
            bool hitL = lc.halfAngle >= 0.0f;
            if (hitL) {
                NodeBox lb = loadNode<64>(nodes, li);
                dl = boxSphereD2Min(lb.pMin, lb.pMax, c);
                hitL = dl <= r2;
                if (hitL) hitL = coneOverlap<DIM>(lc.axis, lc.halfAngle, lc.radius, c, lb.pMin, lb.pMax, dl);
            }
            NodeCone rc = loadCone(nodes, ri);
            bool hitR = rc.halfAngle >= 0.0f;
            if (hitR) {
                NodeBox rb = loadNode<64>(nodes, ri);
                dr = boxSphereD2Min(rb.pMin, rb.pMax, c);
                hitR = dr <= r2;
                if (hitR) hitR = coneOverlap<DIM>(rc.axis, rc.halfAngle, rc.radius, c, rb.pMin, rb.pMax, dr);
            }
            if (hitL && hitR) {
                uint32_t closer = li, other = ri;
                if (dr < dl) { closer = ri; other = li; }
                if (sp + 2 >= kStackDepth) { atomicOr(errorWord, kErrStackOverflow); break; }
                stack[++sp] = other;
                stack[++sp] = closer;
            } else if (hitL || hitR) {
                if (sp + 1 >= kStackDepth) { atomicOr(errorWord, kErrStackOverflow); break; }
                stack[++sp] = hitL ? li : ri;
            }
        }
    }
    return found;
}

}  // namespace fcpwgb
