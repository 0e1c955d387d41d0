// Checkpointed forward and adjoint kernels for Chebyshev degrees 1..5.
#include "adjoint_df.cuh"

namespace tbg {
void register_adjoint_a(CkptFn* c, AdjFn* a, AdjDfFn* d) {
  register_adjoint_degree<2>(c, a, d);  // q = 1
  register_adjoint_degree<3>(c, a, d);  // q = 2
  register_adjoint_degree<4>(c, a, d);  // q = 3
  register_adjoint_degree<5>(c, a, d);  // q = 4
  register_adjoint_degree<6>(c, a, d);  // q = 5
}
}  // namespace tbg
