// Tree kernels instantiated for Chebyshev degrees 1..7.
#include "tree_kernels.cuh"

namespace tbg {
void register_degrees_a(DegreeKernels* table) {
  register_degree<2>(table);  // q = 1
  register_degree<3>(table);  // q = 2
  register_degree<4>(table);  // q = 3
  register_degree<5>(table);  // q = 4
  register_degree<6>(table);  // q = 5
  register_degree<7>(table);  // q = 6
  register_degree<8>(table);  // q = 7
}
}  // namespace tbg
