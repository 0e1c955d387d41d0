// Checkpointed forward and adjoint kernels for Chebyshev degrees 1..5.
#include "adjoint_kernels.cuh"

namespace tbg {
void register_adjoint_a(CkptFn* c, AdjFn* a) {
  register_adjoint_degree<2>(c, a);  // q = 1
  register_adjoint_degree<3>(c, a);  // q = 2
  register_adjoint_degree<4>(c, a);  // q = 3
  register_adjoint_degree<5>(c, a);  // q = 4
  register_adjoint_degree<6>(c, a);  // q = 5
}
}  // namespace tbg
