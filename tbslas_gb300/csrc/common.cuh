// Device-side building blocks of the SL path: Morton keys, leaf lookup,
// Chebyshev recurrences and the triangular tensor Chebyshev sum.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "df64.cuh"
#include "fp64_bits.cuh"
#include "tbslas_gb300.h"

namespace tbg {

// Bits per axis of a point / leaf Morton key.  Leaves may be at most this
// deep.  PVFMM keys points at MAX_DEPTH = 30 bits; for leaves of depth <= 21
// the leaf a point falls in is the same at 21 bits (the low 27 interleaved
// bits of a leaf anchor are zero), so 63-bit keys lose nothing.
constexpr int kKeyBits = 21;
constexpr uint64_t kKeyScale = 1ull << kKeyBits;

// Spread the low 21 bits of v so that bit b lands on bit 3b.
__host__ __device__ inline uint64_t spread3(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

// Interleaved key: inside each level z is the most significant bit, then y,
// then x -- the order of pvfmm::MortonId's comparison and of the leaves'
// post-order (child index x + 2y + 4z).
__host__ __device__ inline uint64_t morton3(uint64_t x, uint64_t y, uint64_t z) {
  return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

// Single periodic wrap of one coordinate, src/tree/tree_functor.h:442-448.
__device__ __forceinline__ double wrap1(double c) {
  if (below_zero(c)) c = c + 1.0;
  if (at_least_one(c)) c = c - 1.0;
  return c;
}

// wrap1 on a point's three coordinates, its FP64 additions issued only when
// some lane of the warp needs them (a predicated-off FP64 instruction still
// takes its slot in the FP64 pipe); wrap1 leaves coordinates in [0, 1) as
// they are, so skipping it there changes nothing.
__device__ __forceinline__ void wrap3(double& x, double& y, double& z) {
  const bool need = !(in_unit_open(x) && in_unit_open(y) && in_unit_open(z));
  if (__any_sync(__activemask(), need)) {
    x = wrap1(x);
    y = wrap1(y);
    z = wrap1(z);
  }
}

// Axis coordinate -> 21-bit integer, floor(c 2^21) (the product is exact, a
// power-of-two scaling) formed from the mantissa and exponent.  The caller
// has checked 0 <= c <= 1 (c < 1 under periodic).  c == 1.0 is shifted into
// the last cell as the reference does for non-periodic trees
// (src/tree/tree_functor.h:464-479).
__device__ __forceinline__ uint64_t quantise(double c) { return floor_scaled(c, kKeyBits); }

// Is the (already wrapped) point inside the domain?  NaN compares false.
__device__ __forceinline__ bool inside(double x, double y, double z, bool periodic) {
  if (periodic) return in_unit_open(x) && in_unit_open(y) && in_unit_open(z);
  return in_unit_closed(x) && in_unit_closed(y) && in_unit_closed(z);
}

// Per-leaf geometry: anchor x, y, z and w = 2*2^depth (the scale that maps
// the leaf onto [-1,1], src/tree/tree_functor.h:286-294).
struct __align__(32) Geom {
  double x, y, z, w;
};
// 2 / w = 2^-depth, the leaf's side (exact, fp64_bits.cuh).
__device__ __forceinline__ double leaf_side(const Geom& g) { return inverse_pow2_times2(g.w); }
__device__ __forceinline__ Geom load_geom(const Geom* p) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return Geom{a.x, a.y, b.x, b.y};
}

// Read-only view of a device tree.
struct TreeView {
  const uint64_t* __restrict__ keys;   // [L] anchor keys, strictly increasing
  const Geom* __restrict__ geom;       // [L]
  const double* __restrict__ coeff;    // [L * stride]
  const float2* __restrict__ coeff2;   // [L * stride] the same, split hi + lo
  const double* __restrict__ cnorm;    // [L * dof] sum of |c| per leaf and component
  const int32_t* __restrict__ table;   // [8^T + 1] coarse-cell -> first leaf
  int64_t L;
  int64_t stride;  // doubles per leaf (dof*Nc rounded up to an even count)
  int T;           // level of the coarse lookup table
  int q;
  int dof;
};

// Index of the leaf containing a point key: the last leaf whose anchor key is
// <= the point key, i.e. the partition std::lower_bound builds over sorted
// point keys in EvalNodesLocal (src/tree/tree_functor.h:193-198).  The coarse
// table narrows the search to the leaves inside one level-T cell.
__device__ __forceinline__ int64_t find_leaf(const TreeView& t, uint64_t key) {
  const uint64_t cell = key >> (3 * (kKeyBits - t.T));
  int64_t lo = __ldg(t.table + cell);
  int64_t hi = __ldg(t.table + cell + 1);
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (__ldg(t.keys + mid) <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// T_0..T_{D-1}(xi); all zero when |xi| > 1 or xi is NaN (pvfmm::cheb_poly as
// called at src/tree/tree_functor.h:328-330).
template <int D>
__device__ __forceinline__ void cheb_T(double xi, double (&T)[D]) {
  const bool ok = abs_at_most_one(xi);
  const double x = ok ? xi : 0.0;
  T[0] = ok ? 1.0 : 0.0;
  if (D > 1) T[1] = x;
  const double x2 = twice(x);
#pragma unroll
  for (int k = 2; k < D; ++k) T[k] = fma(x2, T[k - 1], -T[k - 2]);
}

// Triangular tensor Chebyshev sum of one dof:
//   sum_i tz_i sum_{j<D-i} ty_j sum_{k<D-i-j} c[i][j][k] tx_k
// with the reference's summation order (pvfmm::vec_eval,
// src/tree/tree_functor.h:38-77): each sum starts from +0.0 and adds its
// terms in increasing index by fused multiply-adds.  The first term of each
// sum (T_0 = 1) is formed by fma_t0 with the same bits.  tx/ty/tz as cheb_T
// forms them.  Fully unrolled; c is read with compile-time offsets.
template <int D, class Load>
__device__ __forceinline__ double tri_sum(Load c, const double (&tx)[D], const double (&ty)[D],
                                          const double (&tz)[D]) {
  double u = 0.0;
  int idx = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    double v = 0.0;
#pragma unroll
    for (int j = 0; j < D - i; ++j) {
      double w = fma_t0(tx[0], c(idx));
      ++idx;
#pragma unroll
      for (int k = 1; k < D - i - j; ++k) {
        w = fma(c(idx), tx[k], w);
        ++idx;
      }
      v = j == 0 ? fma_t0(ty[0], w) : fma(ty[j], w, v);
    }
    u = i == 0 ? fma_t0(tz[0], v) : fma(tz[i], v, u);
  }
  return u;
}

struct GlobalLoad {
  const double* __restrict__ p;
  __device__ __forceinline__ double operator()(int i) const { return __ldg(p + i); }
};
struct SharedLoad {
  const double* p;
  __device__ __forceinline__ double operator()(int i) const { return p[i]; }
};

// Evaluate DOF components of a tree at one point.  The point is wrapped in
// place under periodic boundaries (the caller sees the wrapped point, as
// with EvalTree's in-place wrap, src/tree/tree_functor.h:442-448).
// The target whose node values a node-grid output holds for target t: a
// shared upper-face node reads its neighbour's node (the same point) when
// the face map says so and the pass left it unwritten.
__device__ __forceinline__ int64_t node_source(const int32_t* face, int64_t t) {
  if (!face) return t;
  const int32_t f = __ldg(face + t);
  return f >= 0 ? (int64_t)f : t;
}

template <int D, int DOF>
__device__ __forceinline__ void eval_point(const TreeView& t, double& x, double& y, double& z,
                                           bool periodic, double (&out)[DOF]) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  if (periodic) wrap3(x, y, z);
  if (!inside(x, y, z, periodic)) {
#pragma unroll
    for (int l = 0; l < DOF; ++l) out[l] = 0.0;
    return;
  }
  const uint64_t key = morton3(quantise(x), quantise(y), quantise(z));
  const int64_t leaf = find_leaf(t, key);
  const Geom g = load_geom(t.geom + leaf);
  double tx[D], ty[D], tz[D];
  cheb_T<D>((x - g.x) * g.w - 1.0, tx);
  cheb_T<D>((y - g.y) * g.w - 1.0, ty);
  cheb_T<D>((z - g.z) * g.w - 1.0, tz);
  const double* c = t.coeff + leaf * t.stride;
#pragma unroll
  for (int l = 0; l < DOF; ++l) out[l] = tri_sum<D>(GlobalLoad{c + l * NC}, tx, ty, tz);
}

// Double-float evaluation of DOF components at one point, for the fused
// step; `slots` holds 2*D shared-memory elements of this thread (the y and z
// Chebyshev values of tri_sum_df_rows).  m[a] bounds, per axis, the distance
// between this point and the one an all-FP64 computation would have produced
// (0: identical).  Returns true when the lookup is ambiguous -- within m[a] of
// a face of the leaf on some axis, or just outside the domain -- so the caller
// must recompute the target in FP64.  With ERR, err[l] receives a bound on
// |out[l] - out_fp64[l]|: the sums' rounding (df_sum_err<D>() sum|c|, since
// |T_k| <= 1) plus the change of the expansion over the position uncertainty
// (|dT_k/dxi| <= k^2 on [-1,1]).
//
// df_sum_err: worst-case error of the three nested double-float sums relative
// to S = sum |c T T T|, with u = 2^-24.  One df_fma_acc of a row of n terms
// forms each product to 9 u^2 |c t| (two FMA roundings at <= 3u|ct| and 4u|ct|,
// the dropped lo*lo term, the operands' splits) and adds it with an exact
// TwoSum; the low word collects the product and TwoSum errors (|lo_k| <=
// (k+4) u S) and each of its two additions rounds at <= u |lo|, so a row
// carries <= (n^2/2 + 4.5 n + 13) u^2 S, df_norm included.  The i, j, k
// levels add one such term each (the inner errors enter the outer sums with
// weights |T| <= 1), and the FP64 path's own rounding (<= 3 D 2^-53 S) and the
// splits of T and c add < 10 u^2 S.  So |df - fp64| <= (3 (D^2/2 + 4.5 D + 13)
// + 10) 2^-48 S: 2.1e-12 at q = 14.  (Observed errors are ~1e-16 S; the bound
// only sizes the ambiguity margins.)
template <int D>
__host__ __device__ constexpr double df_sum_err() {
  return (3.0 * (0.5 * D * D + 4.5 * D + 13.0) + 10.0) * 0x1p-48;
}

template <int D, int DOF, bool ERR>
__device__ __forceinline__ bool eval_point_df(const TreeView& t, double& x, double& y, double& z,
                                              bool periodic, const double (&m)[3],
                                              double (&out)[DOF], double (&err)[DOF],
                                              ThreadSlots slots) {
  if (periodic) wrap3(x, y, z);
  const double mmax = fmax(m[0], fmax(m[1], m[2]));
  if (!inside(x, y, z, periodic)) {
#pragma unroll
    for (int l = 0; l < DOF; ++l) out[l] = err[l] = 0.0;
    if (mmax == 0.0) return false;
    return x >= -m[0] && x <= 1.0 + m[0] && y >= -m[1] && y <= 1.0 + m[1] && z >= -m[2] &&
           z <= 1.0 + m[2];
  }
  const uint64_t key = morton3(quantise(x), quantise(y), quantise(z));
  const int64_t leaf = find_leaf(t, key);
  const Geom g = load_geom(t.geom + leaf);
  const double xi = (x - g.x) * g.w - 1.0, yi = (y - g.y) * g.w - 1.0, zi = (z - g.z) * g.w - 1.0;
  const bool amb = (m[0] > 0.0 && fabs(xi) >= 1.0 - m[0] * g.w) ||
                   (m[1] > 0.0 && fabs(yi) >= 1.0 - m[1] * g.w) ||
                   (m[2] > 0.0 && fabs(zi) >= 1.0 - m[2] * g.w);
  double T[D];
  df tx[D];
  const ThreadSlots ty = slots, tz{slots.s + D * slots.bs, slots.bs};
  cheb_T<D>(yi, T);
#pragma unroll
  for (int k = 0; k < D; ++k) ty.put(k, df_split_bits(T[k]));
  cheb_T<D>(zi, T);
#pragma unroll
  for (int k = 0; k < D; ++k) tz.put(k, df_split_bits(T[k]));
  cheb_T<D>(xi, T);
#pragma unroll
  for (int k = 0; k < D; ++k) tx[k] = df_split_bits(T[k]);
  df r[DOF];
  tri_sum_df_rows<D, DOF>(t.coeff2 + leaf * t.stride, tx, ty, tz, r);
#pragma unroll
  for (int l = 0; l < DOF; ++l) {
    out[l] = df_to_double(r[l]);
    if (ERR) {
      const double cn = __ldg(t.cnorm + leaf * DOF + l);
      err[l] = cn * (df_sum_err<D>() + (double)((D - 1) * (D - 1)) * g.w * mmax);
    }
  }
  return amb;
}

// The leaf lookup of eval_point_df without the sums: true when (x, y, z) --
// wrapped under periodic boundaries -- lies within m[a] of a face of its leaf
// on some axis, or just outside the domain, so that the FP64 path's lookup
// could differ.
__device__ __forceinline__ bool lookup_ambiguous(const TreeView& t, double x, double y, double z,
                                                 bool periodic, const double (&m)[3]) {
  if (periodic) wrap3(x, y, z);
  if (!inside(x, y, z, periodic)) {
    if (fmax(m[0], fmax(m[1], m[2])) == 0.0) return false;
    return x >= -m[0] && x <= 1.0 + m[0] && y >= -m[1] && y <= 1.0 + m[1] && z >= -m[2] &&
           z <= 1.0 + m[2];
  }
  const int64_t leaf = find_leaf(t, morton3(quantise(x), quantise(y), quantise(z)));
  const Geom g = load_geom(t.geom + leaf);
  const double xi = (x - g.x) * g.w - 1.0, yi = (y - g.y) * g.w - 1.0, zi = (z - g.z) * g.w - 1.0;
  return (m[0] > 0.0 && fabs(xi) >= 1.0 - m[0] * g.w) ||
         (m[1] > 0.0 && fabs(yi) >= 1.0 - m[1] * g.w) ||
         (m[2] > 0.0 && fabs(zi) >= 1.0 - m[2] * g.w);
}

// Position update p = x + s*v of one axis in the double-float step, with its
// uncertainty: mx bounds x's distance from the FP64 path, ev bounds v's.  When
// x is exact and the whole step (plus its uncertainty) is below half an ulp
// of x, both paths round back to x exactly and the result stays exact.
__device__ __forceinline__ void df_update(double s, double v, double ev, double x, double mx,
                                          double& p, double& mp) {
  p = fma(s, v, x);
  const double step = fabs(s) * (fabs(v) + ev);
  if (mx == 0.0 && p == x && step < fabs(x) * 0x1p-54) {
    mp = 0.0;
  } else {
    mp = mx + fabs(s) * ev;
  }
}

// 1-D Chebyshev nodes on [0,1] (new_nodes, src/utils/cheb.h:50-58) passed by
// value to kernels.
struct Nodes1D {
  double x[TBSLAS_MAX_DEGREE + 1];
};

// Device error word bits.
enum : uint32_t {
  kErrBarrierTimeout = 1u << 0,
  kErrBadLeaf = 1u << 1,
  // a coefficient or grid value with |x| >= 2^100 (or not finite) met a
  // double-float split; the double-float results are then meaningless (use
  // TBSLAS_SUMS_FP64)
  kErrDfRange = 1u << 2,
};

__device__ __forceinline__ void check_df_range(double x, uint32_t* err) {
  if (err && !(fabs(x) < 0x1p100)) atomicOr(err, kErrDfRange);
}

}  // namespace tbg
