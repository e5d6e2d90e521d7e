// Wide (branching 4/8) trees with optionally quantised child boxes, derived
// from the transferred binary tree. See wide.cpp / k_wide.cu.
#pragma once

#include <cstdint>
#include <vector>

namespace fcpwgb {

struct WideConfig {
    int branching = 0;   // 0 = traverse the binary tree as transferred (reference order)
    int bits = 32;       // child box precision: 32 (float), 16 or 8 (quantised)
    int blockSize = 256; // threads per block for the wide kernels
    int sortQueries = 0; // reorder queries along a Morton curve before traversal
};

struct WideTree {
    bool valid = false;
    int branching = 0, bits = 32;
    uint64_t builtFromVersion = 0;
    void clear() { valid = false; }
};

}  // namespace fcpwgb
