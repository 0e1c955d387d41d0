// Tree kernels instantiated for Chebyshev degrees 13..13.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_e(DegreeKernels* table) {
  register_degree<14>(table);  // q = 13
}
}  // namespace tbg
