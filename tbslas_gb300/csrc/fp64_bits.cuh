// FP64 operations whose results are formed exactly from the bits of their
// operands with integer instructions.
//
// Every SL kernel here is bound by the FP64 pipe (2 FMA per clock per SM on
// GB300); the integer pipe beside it idles.  So each FP64 instruction that is
// not FP64 arithmetic -- a comparison against 0 or 1, a power-of-two scaling,
// a product by T_0 = 1, a difference of exact small integers -- is formed
// here from the bits instead.  Each function gives the FP64 operation's
// result bit for bit, for every input it is documented for (-0.0,
// subnormals, infinities and NaN included where stated); tests/cpp/
// fp64_bits_check.cpp compares every one against the FP64 operation on the
// host.  Host and device compile the same code.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifndef __CUDACC__
#define TBG_BITS_FN inline
#else
#define TBG_BITS_FN __host__ __device__ __forceinline__
#endif

namespace tbg {

TBG_BITS_FN uint64_t dbits(double c) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(c);
#else
  uint64_t b;
  memcpy(&b, &c, sizeof b);
  return b;
#endif
}
TBG_BITS_FN double from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double c;
  memcpy(&c, &b, sizeof c);
  return c;
#endif
}
TBG_BITS_FN int clz64(uint64_t x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

constexpr uint64_t kBitsOne = 0x3FF0000000000000ull;   // 1.0
constexpr uint64_t kBitsInf = 0x7FF0000000000000ull;   // +inf
constexpr uint64_t kBitsNegZero = 0x8000000000000000ull;
constexpr uint64_t kBitsAbs = 0x7FFFFFFFFFFFFFFFull;
constexpr uint64_t kBitsMant = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kBitsNaN = 0x7FF8000000000000ull;

// ---- comparisons (every input) ---------------------------------------------
// c < 0.0: sign set, not -0.0, not a NaN (bits in (-0.0, -inf]).
TBG_BITS_FN bool below_zero(double c) { return dbits(c) - (kBitsNegZero + 1) < kBitsInf; }
// c >= 1.0: bits in [1.0, +inf].
TBG_BITS_FN bool at_least_one(double c) {
  return dbits(c) - kBitsOne <= 0x4000000000000000ull;
}
// 0 <= c <= 1 (closed) or 0 <= c < 1 (open).
TBG_BITS_FN bool in_unit_closed(double c) {
  const uint64_t b = dbits(c);
  return b <= kBitsOne || b == kBitsNegZero;
}
TBG_BITS_FN bool in_unit_open(double c) {
  const uint64_t b = dbits(c);
  return b < kBitsOne || b == kBitsNegZero;
}
// |c| <= 1 (NaN false).
TBG_BITS_FN bool abs_at_most_one(double c) { return (dbits(c) & kBitsAbs) <= kBitsOne; }

// ---- scalings ----------------------------------------------------------------
// 2x for |x| <= 1 (the Chebyshev recurrence's multiplier): the exponent
// raised by one, or the mantissa shifted for zero and subnormals.
TBG_BITS_FN double twice(double x) {
  const uint64_t b = dbits(x);
  return from_bits((b & kBitsInf) ? b + (1ull << 52)
                                  : (b & kBitsNegZero) | ((b & kBitsAbs) << 1));
}
// 2 / w for w = 2^k, 1 <= k <= 1023 (a leaf's side from its scale 2^(depth+1)).
TBG_BITS_FN double inverse_pow2_times2(double w) {
  return from_bits((2047ull - (dbits(w) >> 52)) << 52);
}
// floor(c 2^bits) for 0 <= c <= 1 (-0.0 included), bits <= 31; c >= 1 gives
// 2^bits - 1 (the Morton quantisation, which puts c = 1 into the last cell).
// The product c 2^bits is exact (a power-of-two scaling), so its floor is the
// mantissa shifted by the exponent.
TBG_BITS_FN uint64_t floor_scaled(double c, int bits) {
  const uint64_t b = dbits(c) & kBitsAbs;  // -0.0 -> +0.0
  if (b >= kBitsOne) return (1ull << bits) - 1;
  const int s = 1075 - bits - (int)(b >> 52);  // c 2^bits = M 2^-s, s >= 53 - bits
  if (s > 52) return 0;                         // c < 2^-bits, zero, subnormal
  return ((b & kBitsMant) | (1ull << 52)) >> s;
}

// ---- products by T_0 (Chebyshev sums) ----------------------------------------
// fma(t0, x, +0.0) for t0 in {+0.0, 1.0} (T_0 as the recurrences form it: 1
// inside [-1, 1], +0 outside), every x: x with -0.0 read as +0.0 when t0 = 1;
// +0.0 (NaN for a non-finite x) when t0 = 0.  The first term of every row of
// a Chebyshev sum is this product, so a row costs one FP64 instruction less.
TBG_BITS_FN double fma_t0(double t0, double x) {
  const uint64_t b = dbits(x);
  if (dbits(t0) != 0) return from_bits(b == kBitsNegZero ? 0ull : b);
  return from_bits((b & kBitsAbs) < kBitsInf ? 0ull : kBitsNaN);
}
// t0 * x for t0 in {+0.0, 1.0}, every x: x when t0 = 1; +-0 with x's sign
// (NaN for a non-finite x) when t0 = 0.
TBG_BITS_FN double mul_t0(double t0, double x) {
  const uint64_t b = dbits(x);
  if (dbits(t0) != 0) return x;
  return from_bits((b & kBitsAbs) < kBitsInf ? (b & kBitsNegZero) : kBitsNaN);
}

// ---- the tricubic stencil of a power-of-two periodic grid --------------------
// ix 2^-nl as a double, 0 <= ix < 2^31 (the node coordinate ix h, h = 2^-nl).
TBG_BITS_FN double grid_coord_pow2(int64_t ix, int nl) {
  if (ix == 0) return 0.0;
  const int p = 63 - clz64((uint64_t)ix);
  const uint64_t m = ((uint64_t)ix << (52 - p)) & kBitsMant;
  return from_bits(((uint64_t)(1023 + p - nl) << 52) | m);
}

// Stencil base and offset of one coordinate x in [0, 1) (-0.0 included) on a
// periodic grid of N = 2^nl nodes: p = x N, g = floor(p) - 1, t = p - g in
// [1, 2] -- the values p - (double)g gives in FP64: x N is exact; t is exact
// for p >= 1, and for p < 1 (the first cell) it is 1 + p rounded to nearest
// even, formed here from the bits of p.
TBG_BITS_FN void grid_split_pow2(double x, int nl, int& g, double& t) {
  const uint64_t b = dbits(x);
  const uint64_t M = (b & kBitsMant) | (1ull << 52);  // x normal: p = M 2^-s
  const int s = 1075 - nl - (int)(b >> 52);
  if ((b << 1) == 0 || s > 52) {  // +-0, or p < 1 (subnormal x included)
    g = -1;
    // 1 + p = 1 + q 2^-52 with q = p 2^52 = M 2^-(s - 52) rounded to nearest
    // even (M 2^-sh with sh = s - 52 >= 1; a subnormal or zero x gives 0)
    uint64_t q = 0;
    const int sh = s - 52;
    if ((b & kBitsInf) != 0 && sh < 64) {
      q = M >> sh;
      const uint64_t rem = M & ((1ull << sh) - 1), half = 1ull << (sh - 1);
      if (rem > half || (rem == half && (q & 1))) ++q;
    }
    t = from_bits((1023ull << 52) + q);  // q = 2^52 carries into the exponent: t = 2
    return;
  }
  g = (int)(M >> s) - 1;
  const uint64_t frac = s > 0 ? (M & ((1ull << s) - 1)) : 0ull;
  t = from_bits((1023ull << 52) | (frac << (52 - s)));
}

// Cubic Lagrange weights at offset t from the stencil base, formed exactly as
// the reference does (denominators by repeated division, then the product of
// (t - l) over l != k in increasing l): src/tree/tree_functor.h:93-99,
// :126-135.
TBG_BITS_FN void lagrange4(double t, double (&w)[4]) {
  const double den[4] = {-1.0 / 6.0, 0.5, -0.5, 1.0 / 6.0};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double m = den[k];
#pragma unroll
    for (int l = 0; l < 4; ++l)
      if (k != l) m *= (t - (double)l);
    w[k] = m;
  }
}

// g 2^-52 as a double for 0 < g <= 2^53 (exact: g has at most 53 bits), with
// the sign bit set when neg.
TBG_BITS_FN double scaled_mantissa(uint64_t g, bool neg) {
  const int p = 63 - clz64(g);  // leading bit, <= 53
  const uint64_t m = p <= 52 ? (g << (52 - p)) & kBitsMant : 0ull;
  return from_bits((neg ? kBitsNegZero : 0ull) | ((uint64_t)(1023 + p - 52) << 52) | m);
}

// lagrange4 for an offset t in [1, 2) (a power-of-two grid's): the same
// products in the same order, with t - 1, t - 2, t - 3 and the exact
// halvings +-t/2 formed from the mantissa of t (each of those FP64
// operations is exact, so the values are the same).  Other offsets (t
// rounded up to 2 in the first cell) take lagrange4.
TBG_BITS_FN void lagrange4_unit(double t, double (&w)[4]) {
  const uint64_t b = dbits(t);
  if ((b >> 52) != 1023) {
    lagrange4(t, w);
    return;
  }
  const uint64_t f = b & kBitsMant;
  const double d1 = f ? scaled_mantissa(f, false) : 0.0;      // t - 1 in [0, 1)
  const double d2 = scaled_mantissa((1ull << 52) - f, true);  // t - 2 in [-1, 0)
  const double d3 = scaled_mantissa((1ull << 53) - f, true);  // t - 3 in [-2, -1)
  const uint64_t hb = b - (1ull << 52);                        // t / 2
  const double h = from_bits(hb);
  const double hn = from_bits(hb | kBitsNegZero);
  w[0] = ((-1.0 / 6.0 * d1) * d2) * d3;
  w[1] = (h * d2) * d3;
  w[2] = (hn * d1) * d3;
  w[3] = ((1.0 / 6.0 * t) * d1) * d2;
}

}  // namespace tbg
