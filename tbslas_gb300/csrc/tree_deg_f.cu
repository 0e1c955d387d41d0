// Tree kernels instantiated for Chebyshev degrees 14..14.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_f(DegreeKernels* table) {
  register_degree<15>(table);  // q = 14
}
}  // namespace tbg
