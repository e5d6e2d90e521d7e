// Wide (branching 2/4/8) trees with 32-bit, 16-bit or 8-bit child boxes,
// derived from the transferred binary tree (wide_build.cu builds them on the
// host, k_wide.cu traverses and re-quantises them on the device).
//
// Node record (size a multiple of 16 B, array 16 B aligned):
//   [header, quantised only: float origin[3]; uint8 exponent[3] (biased by 127); uint8 nChildren]
//   uint32 ref[W]      inner child: wide node index; leaf child: first primitive
//   uint8  cnt[W]      0 = inner child, 1..15 = leaf primitive count, 255 = empty slot
//   bounds             lo[axis][W] then hi[axis][W]: float, uint16 or uint8
// A quantised child box is origin + q * 2^exponent per axis, evaluated as
// fmaf(q, 2^e, origin); the quantiser rounds lo down / hi up and checks every
// bound with that same fmaf, so each dequantised box contains its child.
#pragma once

#include <cstdint>
#include <vector>

namespace fcpwgb {

constexpr uint8_t kWideEmpty = 255;
constexpr int kWideStack = 128;  // per-thread traversal stack entries of the wide kernels

struct WideConfig {
    int branching = 0;   // 0 = traverse the binary tree as transferred (reference order)
    int bits = 32;       // child box precision: 32 (float), 16 or 8 (quantised)
    int blockSize = 128; // threads per block
    int sortQueries = 1; // reorder queries by spatial cell before traversal
    int persistent = 1;  // persistent blocks fetching query chunks from a work counter
    int precise = 1;     // refine the winning primitive's distance to within 1e-6 of FP64
    int packet = 0;      // traverse the 32 queries of a warp as one packet
    int leafSize = 0;    // > 0: binary subtrees of at most this many primitives collapse into one leaf
    int shortStack = 16; // traversal stack entries per thread in shared memory (thread schedules): 0 or 16
    int lanes = 1;       // lanes answering one query together (1, 2, 4 or 8)
};

constexpr int wideHeaderBytes(int bits) { return bits == 32 ? 0 : 16; }
constexpr int wideCntOffset(int W, int bits) { return wideHeaderBytes(bits) + 4 * W; }
constexpr int wideBoundsOffset(int W, int bits) { return ((wideCntOffset(W, bits) + W) + 3) / 4 * 4; }
constexpr int wideNodeBytes(int W, int bits) {
    return (wideBoundsOffset(W, bits) + 6 * W * (bits / 8) + 15) / 16 * 16;
}

// host-side result of collapsing a binary tree
struct WideHost {
    int W = 4, bits = 32;
    uint32_t nNodes = 0, depth = 0;
    std::vector<unsigned char> nodes;   // nNodes * wideNodeBytes(W, bits)
    std::vector<int32_t> childBinary;   // nNodes * W: binary node behind every slot (-1 = empty)
};

// Collapses a binary pre-order tree (nPrims/offset per node, boxes as
// pMin[3], pMax[3] per node) into a W-wide tree: starting from the two
// children of a binary inner node, the inner child of largest surface area is
// replaced by its two children until W children are reached (the
// max-surface-area rule of the reference's Mbvh collapse,
// include/fcpw/aggregates/mbvh.inl:57-147). Returns false if a leaf cannot
// be encoded (more than 15 primitives) or the wide stack could overflow.
// maxLeafSize > 0 also turns every binary subtree of at most that many
// primitives (which the pre-order SAH build stores contiguously) into one
// wide leaf; 0 keeps the binary leaves as they are.
bool buildWideTree(int W, int bits, const std::vector<uint32_t> &nPrims, const std::vector<uint32_t> &offsets,
                   const std::vector<float> &boxes, WideHost &out, int maxLeafSize = 0);

// what a scene keeps about its derived wide tree (buffers live in the scene)
struct WideTree {
    bool valid = false;
    int branching = 0, bits = 32, leafSize = 0;
    uint32_t nNodes = 0, depth = 0;
    uint64_t builtFromVersion = 0;
    void clear() { valid = false; }
};

}  // namespace fcpwgb
