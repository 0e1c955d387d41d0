// Tree kernels instantiated for Chebyshev degrees 8..9.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_b(DegreeKernels* table) {
  register_degree<9>(table);  // q = 8
  register_degree<10>(table);  // q = 9
}
}  // namespace tbg
