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

// Split of an FP64 value into hi + lo with integer operations only (no FP64
// pipe, which runs at 1/72 of the FP32 rate): hi = x with its significand
// truncated to 24 bits, lo = the remaining 29 significand bits rounded to a
// float.  |x - hi - lo| <= 2^-48 |x|; values below 2^-74 lose lo and values
// below 2^-126 become 0 (absolute error < 2^-97, resp. 2^-126 -- far below
// the sums' error bound).  |x| >= 2^127, inf and NaN take the float
// conversion (inf / NaN as in FP64; callers flag |x| >= 2^100 as outside the
// double-float range).
__device__ __forceinline__ df df_split_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  if (e < 897u) return df{0.f, 0.f};
  if (e > 1149u) return df{__double2float_rn(x), 0.f};  // exponent field 254 at most
  const float hi = __uint_as_float(sign | ((e - 896u) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
  float lo = 0.f;
  if (e >= 949u) {
    const float scale = __uint_as_float((e - 948u) << 23);  // 2^(e - 1075)
    lo = __uint_as_float(__float_as_uint(__fmul_rn(__uint2float_rn((unsigned)(b & 0x1fffffffu)),
                                                   scale)) | sign);
  }
  return df{hi, lo};
}

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

// One thread's array in shared memory: element k at s[k * bs] (bs = the
// block size), so a warp's accesses to one element are conflict-free.
struct ThreadSlots {
  float2* s;
  int bs;
  __device__ __forceinline__ df get(int k) const {
    const float2 v = s[k * bs];
    return df{v.x, v.y};
  }
  __device__ __forceinline__ void put(int k, df a) const { s[k * bs] = make_float2(a.hi, a.lo); }
};

// The triangular sum with the i and j loops rolled: the unrolled form is
// ~13 instructions per term x Nc terms per component (35K instructions for a
// velocity and a concentration evaluation at q = 14), far beyond the
// instruction caches, so warps stalled on instruction fetch.  Here the code
// is one row of at most D terms: each (i, j) row of n = D-i-j coefficients
// enters the unrolled sequence k = n-1 .. 0 through a switch (one indexed
// jump), tx stays in registers, ty_j and tz_i come from shared memory.  The
// DOF components share the row's T values and form independent chains.
#define TBG_DF_TERM(K)                                                           \
  case (K) + 1:                                                                  \
    if constexpr ((K) < D) {                                                     \
      _Pragma("unroll") for (int l = 0; l < DOF; ++l)                            \
          df_fma_acc(w[l], ld(l * NC + idx + (K)), tx[(K) < D ? (K) : 0]);       \
    }                                                                            \
    [[fallthrough]];

template <int D, int DOF>
__device__ __forceinline__ void tri_sum_df_rows(const float2* __restrict__ c, const df (&tx)[D],
                                                ThreadSlots ty, ThreadSlots tz, df (&out)[DOF]) {
  static_assert(D >= 1 && D <= 17, "degree above 16");
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  const GlobalLoadDF ld{c};
  df u[DOF];
#pragma unroll
  for (int l = 0; l < DOF; ++l) u[l] = df{0.f, 0.f};
  int idx = 0;
#pragma unroll 1
  for (int i = 0; i < D; ++i) {
    df v[DOF];
#pragma unroll
    for (int l = 0; l < DOF; ++l) v[l] = df{0.f, 0.f};
#pragma unroll 1
    for (int j = 0; j < D - i; ++j) {
      const int n = D - i - j;
      df w[DOF];
#pragma unroll
      for (int l = 0; l < DOF; ++l) w[l] = df{0.f, 0.f};
      switch (n) {
        TBG_DF_TERM(16)
        TBG_DF_TERM(15)
        TBG_DF_TERM(14)
        TBG_DF_TERM(13)
        TBG_DF_TERM(12)
        TBG_DF_TERM(11)
        TBG_DF_TERM(10)
        TBG_DF_TERM(9)
        TBG_DF_TERM(8)
        TBG_DF_TERM(7)
        TBG_DF_TERM(6)
        TBG_DF_TERM(5)
        TBG_DF_TERM(4)
        TBG_DF_TERM(3)
        TBG_DF_TERM(2)
        TBG_DF_TERM(1)
        TBG_DF_TERM(0)
        default:
          break;
      }
      idx += n;
      const df yj = ty.get(j);
#pragma unroll
      for (int l = 0; l < DOF; ++l) df_fma_acc(v[l], yj, df_norm(w[l]));
    }
    const df zi = tz.get(i);
#pragma unroll
    for (int l = 0; l < DOF; ++l) df_fma_acc(u[l], zi, df_norm(v[l]));
  }
#pragma unroll
  for (int l = 0; l < DOF; ++l) out[l] = df_norm(u[l]);
}
#undef TBG_DF_TERM

}  // namespace tbg
