// Double-float ("df64") arithmetic on the FP32 pipe for the triangular
// Chebyshev sums of the fused SL step.
//
// GB300 executes FP64 at 1/72 of its FP32 rate (1.06 vs 76.7 TFLOP/s
// measured), so the bulk of the step -- the Nc-term sums -- runs as pairs of
// floats: a value is hi + lo with |lo| <= ulp(hi)/2 (48 significant bits).
// Products are formed exactly with an FMA (Dekker/Ogita-Rump-Oishi error-free
// transformations: TwoProduct via FMA, Knuth's TwoSum), partial sums keep
// their rounding errors in lo, and every level of the sum is renormalised.
// All float operations use the _rn intrinsics, which the compiler never
// contracts or reassociates (the transformations rely on exact rounding).
//
// Relative error per term ~2^-47 of the term; the Chebyshev series of the
// advected fields have decaying coefficients, so the result carries ~1e-14
// relative error -- below the 1e-12 tolerance of the step, far above what a
// leaf choice could tolerate, which is why coordinates and leaf lookups stay
// FP64 and near-face points are recomputed in FP64.
#pragma once

#include <cuda_runtime.h>

namespace tbg {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_from_double(double x) {
  const float h = __double2float_rn(x);
  return df{h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df df_norm(df a) {
  const float s = __fadd_rn(a.hi, a.lo);
  return df{s, __fsub_rn(a.lo, __fsub_rn(s, a.hi))};
}

// acc += a * b (a, b normalised; acc's lo collects the errors, normalised by
// the caller once per sum).
__device__ __forceinline__ void df_fma_acc(df& acc, df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float s = __fadd_rn(acc.hi, p);
  const float v = __fsub_rn(s, acc.hi);
  const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, v)), __fsub_rn(p, v));
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, err));
  acc.hi = s;
}

struct GlobalLoadDF {
  const float2* __restrict__ p;
  __device__ __forceinline__ df operator()(int i) const {
    const float2 v = __ldg(p + i);
    return df{v.x, v.y};
  }
};

// sum_i tz_i sum_{j<D-i} ty_j sum_{k<D-i-j} c[i][j][k] tx_k in double-float,
// same nesting as tri_sum.
template <int D, class Load>
__device__ __forceinline__ df tri_sum_df(Load c, const df (&tx)[D], const df (&ty)[D],
                                         const df (&tz)[D]) {
  df u{0.f, 0.f};
  int idx = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    df v{0.f, 0.f};
#pragma unroll
    for (int j = 0; j < D - i; ++j) {
      df w{0.f, 0.f};
#pragma unroll
      for (int k = 0; k < D - i - j; ++k) {
        df_fma_acc(w, c(idx), tx[k]);
        ++idx;
      }
      df_fma_acc(v, ty[j], df_norm(w));
    }
    df_fma_acc(u, tz[i], df_norm(v));
  }
  return df_norm(u);
}

}  // namespace tbg
