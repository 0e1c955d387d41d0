// Adjoint kernels for Chebyshev degrees 9..10.
#include "adjoint_df.cuh"

namespace tbg {
void register_adjoint_c(AdjFn* a, AdjDfFn* d, JacStepFn* j) {
  register_adjoint_degree<10>(a, d, j);  // q = 9
  register_adjoint_degree<11>(a, d, j);  // q = 10
}
}  // namespace tbg
