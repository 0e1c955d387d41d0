// Checkpointed forward and adjoint kernels for Chebyshev degrees 9..10.
#include "adjoint_df.cuh"

namespace tbg {
void register_adjoint_c(CkptFn* c, AdjFn* a, AdjDfFn* d) {
  register_adjoint_degree<10>(c, a, d);  // q = 9
  register_adjoint_degree<11>(c, a, d);  // q = 10
}
}  // namespace tbg
