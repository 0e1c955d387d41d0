// Adjoint kernels for Chebyshev degrees 1..5.
#include "adjoint_df.cuh"

namespace tbg {
void register_adjoint_a(AdjFn* a, AdjDfFn* d, JacStepFn* j) {
  register_adjoint_degree<2>(a, d, j);  // q = 1
  register_adjoint_degree<3>(a, d, j);  // q = 2
  register_adjoint_degree<4>(a, d, j);  // q = 3
  register_adjoint_degree<5>(a, d, j);  // q = 4
  register_adjoint_degree<6>(a, d, j);  // q = 5
}
}  // namespace tbg
