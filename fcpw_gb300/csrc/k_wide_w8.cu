// Instantiation of the wide-tree kernels for branching factor 8 (see k_wide.cuh).
#include "k_wide.cuh"

namespace fcpwgb {
FCPWGB_WIDE_INSTANTIATE(8)
}  // namespace fcpwgb
