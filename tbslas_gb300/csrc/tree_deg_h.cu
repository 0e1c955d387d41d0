// Tree kernels instantiated for Chebyshev degrees 16..16.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_h(DegreeKernels* table) {
  register_degree<17>(table);  // q = 16
}
}  // namespace tbg
