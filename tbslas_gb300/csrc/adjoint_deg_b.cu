// Checkpointed forward and adjoint kernels for Chebyshev degrees 6..8.
#include "adjoint_df.cuh"

namespace tbg {
void register_adjoint_b(CkptFn* c, AdjFn* a, AdjDfFn* d) {
  register_adjoint_degree<7>(c, a, d);  // q = 6
  register_adjoint_degree<8>(c, a, d);  // q = 7
  register_adjoint_degree<9>(c, a, d);  // q = 8
}
}  // namespace tbg
