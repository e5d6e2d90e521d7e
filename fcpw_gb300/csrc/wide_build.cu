// Host collapse of the binary tree into a W-wide tree with quantised child
// boxes (see wide.h for the record layout).
#include <algorithm>
#include <cstring>

#include "wide_common.cuh"

namespace fcpwgb {

namespace {

struct Collapser {
    int W, bits;
    const std::vector<uint32_t> &nP, &off;
    const std::vector<float> &box;
    WideHost &out;
    bool ok = true;
    size_t nodeBytes;
    uint32_t maxLeaf = 0;                   // > 0: subtrees of at most this many primitives become one leaf
    std::vector<uint32_t> subCount, subFirst;  // primitives under a binary node, first of them
    std::vector<char> subContiguous;        // they form one range subFirst .. subFirst + subCount

    // primitive count and range of every binary subtree (pre-order: children after their parent)
    void summarise() {
        const size_t n = nP.size();
        subCount.assign(n, 0);
        subFirst.assign(n, 0);
        subContiguous.assign(n, 1);
        std::vector<uint32_t> subEnd(n, 0);
        for (size_t i = n; i-- > 0;) {
            if (nP[i] > 0) {
                subCount[i] = nP[i];
                subFirst[i] = off[i];
                subEnd[i] = off[i] + nP[i];
            } else {
                uint32_t l = (uint32_t)i + 1, r = (uint32_t)i + off[i];
                subCount[i] = subCount[l] + subCount[r];
                subFirst[i] = std::min(subFirst[l], subFirst[r]);
                subEnd[i] = std::max(subEnd[l], subEnd[r]);
                subContiguous[i] = subContiguous[l] && subContiguous[r] && subEnd[i] - subFirst[i] == subCount[i];
            }
        }
    }
    // a binary node that becomes a leaf slot of the wide tree
    bool leafLike(uint32_t b) const {
        if (nP[b] > 0) return true;
        return maxLeaf > 0 && subContiguous[b] && subCount[b] <= maxLeaf;
    }

    float area(uint32_t b) const {
        const float *p = &box[(size_t)b * 6];
        float ex = p[3] - p[0], ey = p[4] - p[1], ez = p[5] - p[2];
        return 2.0f * (ex * ey + ey * ez + ez * ex);
    }

    // returns the wide node index built for binary inner node b
    uint32_t build(uint32_t b, uint32_t depth) {
        uint32_t idx = out.nNodes++;
        out.depth = std::max(out.depth, depth + 1);
        out.nodes.resize((size_t)out.nNodes * nodeBytes, 0);
        out.childBinary.resize((size_t)out.nNodes * W, -1);

        std::vector<uint32_t> kids;
        if (leafLike(b)) {
            kids.push_back(b);  // a leaf root
        } else {
            kids.push_back(b + 1);
            kids.push_back(b + off[b]);
            while ((int)kids.size() < W) {
                int best = -1;
                float bestA = -1.0f;
                for (size_t i = 0; i < kids.size(); i++) {
                    if (leafLike(kids[i])) continue;
                    float a = area(kids[i]);
                    if (a > bestA) { bestA = a; best = (int)i; }
                }
                if (best < 0) break;
                uint32_t k = kids[best];
                kids[best] = k + 1;
                kids.insert(kids.begin() + best + 1, k + off[k]);
            }
        }

        float lo[8 * 3], hi[8 * 3];
        bool valid[8];
        uint32_t ref[8];
        uint8_t cnt[8];
        for (int c = 0; c < W; c++) {
            valid[c] = c < (int)kids.size();
            ref[c] = 0;
            cnt[c] = kWideEmpty;
            for (int a = 0; a < 3; a++) { lo[c * 3 + a] = 0.0f; hi[c * 3 + a] = 0.0f; }
        }
        for (size_t c = 0; c < kids.size(); c++) {
            uint32_t k = kids[c];
            for (int a = 0; a < 3; a++) {
                lo[c * 3 + a] = box[(size_t)k * 6 + a];
                hi[c * 3 + a] = box[(size_t)k * 6 + 3 + a];
            }
            out.childBinary[(size_t)idx * W + c] = (int32_t)k;
            if (leafLike(k)) {
                uint32_t first = nP[k] > 0 ? off[k] : subFirst[k], count = nP[k] > 0 ? nP[k] : subCount[k];
                if (count > 15 || first >= (1u << 27)) ok = false;
                ref[c] = first;
                cnt[c] = (uint8_t)std::min<uint32_t>(count, 15);
            } else {
                ref[c] = build(k, depth + 1);
                cnt[c] = 0;
            }
        }
        unsigned char *rec = out.nodes.data() + (size_t)idx * nodeBytes;
        std::memcpy(rec + wideHeaderBytes(bits), ref, 4 * W);
        std::memcpy(rec + wideCntOffset(W, bits), cnt, W);
        bool q = true;
        switch (W * 100 + bits) {
            case 232: q = quantizeWideNode<2, 32>(lo, hi, valid, rec); break;
            case 216: q = quantizeWideNode<2, 16>(lo, hi, valid, rec); break;
            case 208: q = quantizeWideNode<2, 8>(lo, hi, valid, rec); break;
            case 432: q = quantizeWideNode<4, 32>(lo, hi, valid, rec); break;
            case 416: q = quantizeWideNode<4, 16>(lo, hi, valid, rec); break;
            case 408: q = quantizeWideNode<4, 8>(lo, hi, valid, rec); break;
            case 832: q = quantizeWideNode<8, 32>(lo, hi, valid, rec); break;
            case 816: q = quantizeWideNode<8, 16>(lo, hi, valid, rec); break;
            case 808: q = quantizeWideNode<8, 8>(lo, hi, valid, rec); break;
            default: q = false;
        }
        if (!q) ok = false;
        return idx;
    }
};

}  // namespace

bool buildWideTree(int W, int bits, const std::vector<uint32_t> &nPrims, const std::vector<uint32_t> &offsets,
                   const std::vector<float> &boxes, WideHost &out, int maxLeafSize) {
    out = WideHost();
    out.W = W;
    out.bits = bits;
    if (!(W == 2 || W == 4 || W == 8) || !(bits == 8 || bits == 16 || bits == 32) || nPrims.empty()) return false;
    if (maxLeafSize < 0 || maxLeafSize > 15) return false;
    Collapser c{W, bits, nPrims, offsets, boxes, out};
    c.nodeBytes = (size_t)wideNodeBytes(W, bits);
    c.maxLeaf = (uint32_t)maxLeafSize;
    if (c.maxLeaf > 0) c.summarise();
    out.nodes.reserve((size_t)nPrims.size() * c.nodeBytes / std::max(1, W - 1) + c.nodeBytes);
    c.build(0, 0);
    // the per-thread stack holds at most (W - 1) entries per level plus one
    if ((uint64_t)(W - 1) * out.depth + 2 > (uint64_t)kWideStack) c.ok = false;
    if (!c.ok) {
        out = WideHost();
        return false;
    }
    return true;
}

}  // namespace fcpwgb
