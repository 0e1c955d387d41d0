// Tree kernels instantiated for Chebyshev degrees 15..15.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_g(DegreeKernels* table) {
  register_degree<16>(table);  // q = 15
}
}  // namespace tbg
