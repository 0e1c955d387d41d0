// Tree kernels instantiated for Chebyshev degrees 10..11.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_c(DegreeKernels* table) {
  register_degree<11>(table);  // q = 10
  register_degree<12>(table);  // q = 11
}
}  // namespace tbg
