// Time-dependent velocity step kernels for Chebyshev degrees 1..9, and the
// coefficient blend of the fast path.
#include "tv_kernels.cuh"

namespace tbg {

namespace {
struct BlendArgs {
  const double* c[kTvMaxTrees];
  double w[kTvMaxTrees];
};

__global__ void k_blend_coeffs(const BlendArgs b, int m, int64_t n, double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < m; ++k) s = fma(b.w[k], __ldg(b.c[k] + i), s);
  out[i] = s;
}
}  // namespace

void launch_blend_coeffs(const double* const* c, const double* w, int m, int64_t n, double* out,
                         cudaStream_t s) {
  BlendArgs b{};
  for (int k = 0; k < m; ++k) {
    b.c[k] = c[k];
    b.w[k] = w[k];
  }
  if (n > 0) k_blend_coeffs<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, m, n, out);
}

void register_tv_a(TvFn* table) {
  table[1] = &launch_semilag_tv<2>;
  table[2] = &launch_semilag_tv<3>;
  table[3] = &launch_semilag_tv<4>;
  table[4] = &launch_semilag_tv<5>;
  table[5] = &launch_semilag_tv<6>;
  table[6] = &launch_semilag_tv<7>;
  table[7] = &launch_semilag_tv<8>;
  table[8] = &launch_semilag_tv<9>;
  table[9] = &launch_semilag_tv<10>;
}
}  // namespace tbg
