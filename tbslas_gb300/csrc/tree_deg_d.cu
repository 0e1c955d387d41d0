// Tree kernels instantiated for Chebyshev degrees 12..12.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_d(DegreeKernels* table) {
  register_degree<13>(table);  // q = 12
}
}  // namespace tbg
