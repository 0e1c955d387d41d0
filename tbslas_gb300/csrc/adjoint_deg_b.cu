// Checkpointed forward and adjoint kernels for Chebyshev degrees 6..8.
#include "adjoint_kernels.cuh"

namespace tbg {
void register_adjoint_b(CkptFn* c, AdjFn* a) {
  register_adjoint_degree<7>(c, a);  // q = 6
  register_adjoint_degree<8>(c, a);  // q = 7
  register_adjoint_degree<9>(c, a);  // q = 8
}
}  // namespace tbg
