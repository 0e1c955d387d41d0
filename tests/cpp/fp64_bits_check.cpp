// Checks every function of tbslas_gb300/csrc/fp64_bits.cuh against the FP64
// operation it stands for, on the host: special values (+-0, subnormals,
// +-inf, NaN of either sign, the neighbours of 0, 1, 2^-k) and seeded random
// inputs (random bit patterns and values in the functions' ranges).  Prints
// "cases N mismatches M" and exits non-zero on a mismatch.
//
// Built with -ffp-contract=off, so each FP64 reference expression below is
// the single IEEE operation it names (and lagrange4's products stay
// products).
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "fp64_bits.cuh"

using namespace tbg;

static long g_cases = 0, g_bad = 0;

static bool same(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return std::isnan(a) && std::isnan(b);
  return dbits(a) == dbits(b);  // signed zeros included
}

static void expect(bool ok, const char* what, double x) {
  ++g_cases;
  if (!ok && g_bad++ < 10) std::printf("mismatch %s at %a\n", what, x);
}

static std::vector<double> specials() {
  std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, -2.0,
                           INFINITY, -INFINITY, NAN, -NAN,
                           5e-324, -5e-324, 2.2250738585072014e-308, -2.2250738585072014e-308,
                           2.225073858507201e-308, 1e-300, -1e-300, 1e300, -1e300};
  for (int k = 0; k <= 60; ++k) {
    const double p = std::ldexp(1.0, -k);
    for (double x : {p, std::nextafter(p, 0.0), std::nextafter(p, 2.0)}) {
      v.push_back(x);
      v.push_back(-x);
      v.push_back(1.0 - x);
    }
  }
  v.push_back(std::nextafter(1.0, 2.0));
  v.push_back(std::nextafter(1.0, 0.0));
  return v;
}

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> unit(0.0, 1.0), sym(-1.0, 1.0);
  std::vector<double> xs = specials();
  for (int i = 0; i < 2000000; ++i) {
    const uint64_t r = rng();
    xs.push_back(from_bits(r));
    xs.push_back(unit(rng));
    xs.push_back(sym(rng));
    xs.push_back(std::ldexp(unit(rng), -(int)(r % 80)));
  }

  for (double c : xs) {
    expect(below_zero(c) == (c < 0.0), "below_zero", c);
    expect(at_least_one(c) == (c >= 1.0), "at_least_one", c);
    expect(in_unit_closed(c) == (c >= 0.0 && c <= 1.0), "in_unit_closed", c);
    expect(in_unit_open(c) == (c >= 0.0 && c < 1.0), "in_unit_open", c);
    expect(abs_at_most_one(c) == (std::fabs(c) <= 1.0), "abs_at_most_one", c);
    if (std::fabs(c) <= 1.0) expect(same(twice(c), 2.0 * c), "twice", c);
    if (c >= 0.0 && c <= 1.0) {
      const uint64_t want = c >= 1.0 ? (1ull << 21) - 1 : (uint64_t)(c * 2097152.0);
      expect(floor_scaled(c, 21) == want, "floor_scaled", c);
    }
    for (double t0 : {0.0, 1.0}) {
      expect(same(fma_t0(t0, c), std::fma(t0, c, 0.0)), "fma_t0", c);
      expect(same(mul_t0(t0, c), t0 * c), "mul_t0", c);
    }
  }
  // leaf sides 2 / 2^(depth+1)
  for (int d = 0; d <= 30; ++d) {
    const double w = std::ldexp(2.0, d);
    expect(same(inverse_pow2_times2(w), 2.0 / w), "inverse_pow2_times2", w);
  }
  // node coordinates and stencil splits of periodic 2^nl grids
  for (int nl = 0; nl <= 12; ++nl) {
    const int N = 1 << nl;
    const double h = 1.0 / N;
    for (int64_t ix = 0; ix < N; ++ix)
      expect(same(grid_coord_pow2(ix, nl), (double)ix * h), "grid_coord_pow2", (double)ix);
  }
  std::vector<double> offs;
  for (int i = 0; i < 1500000; ++i) offs.push_back(unit(rng));
  for (double x : specials())
    if (x >= 0.0 && x < 1.0) offs.push_back(x);
  offs.push_back(-0.0);
  offs.push_back(std::nextafter(1.0 / 256, 0.0) * (1.0 - 0x1p-53));
  // first-cell offsets at ties: p = x N = m 2^-53 for odd m (1 + p halfway
  // between two doubles), placed below each grid's 1 / N later
  std::vector<double> tie_p;
  for (int i = 0; i < 200000; ++i)
    tie_p.push_back(std::ldexp((double)((rng() >> 11) | 1ull), -53));
  for (int i = 0; i < 60; ++i) tie_p.push_back(std::ldexp(1.0, -i - 1) + 0x1p-53);
  for (int nl : {1, 4, 8, 10}) {
    const double N = (double)(1 << nl);
    std::vector<double> xs_nl = offs;
    for (double p : tie_p) xs_nl.push_back(p / N);  // exact: a power-of-two scaling
    for (double x : xs_nl) {
      int g = 0;
      double t = 0.0;
      grid_split_pow2(x, nl, g, t);
      const double p = x * N;
      const int64_t gref = (int64_t)p - 1;
      const double tref = p - (double)gref;
      expect(g == gref && same(t, tref), "grid_split_pow2", x);
      double w[4], wref[4];
      lagrange4_unit(t, w);
      const double den[4] = {-1.0 / 6.0, 0.5, -0.5, 1.0 / 6.0};
      for (int k = 0; k < 4; ++k) {
        double m = den[k];
        for (int l = 0; l < 4; ++l)
          if (k != l) m *= (t - (double)l);
        wref[k] = m;
      }
      for (int k = 0; k < 4; ++k) expect(same(w[k], wref[k]), "lagrange4_unit", t);
    }
  }
  std::printf("cases %ld mismatches %ld\n", g_cases, g_bad);
  return g_bad ? 1 : 0;
}
