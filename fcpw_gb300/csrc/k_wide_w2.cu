// Instantiation of the wide-tree kernels for branching factor 2 (see k_wide.cuh).
#include "k_wide.cuh"

namespace fcpwgb {
FCPWGB_WIDE_INSTANTIATE(2)
}  // namespace fcpwgb
