// Tricubic regular-grid path: the interpolant tbslas::fast_interp
// (src/tree/tree_functor.h:89-153) and a fused SL step on the grid (every node
// a target, RK2 through the interpolated velocity, interpolated concentration
// at the departure point).
//
// Grid layout as the reference: SoA, vals[x + N(y + N z) + k N^3].
//  FREESPACE: nodes i/(N-1); stencil base floor(x(N-1))-1 clamped to
//             [0, N-4]; points outside [0,1]^3 give 0 (the reference's form).
//  PERIODIC:  nodes i/N on [0,1); the query is wrapped once (as EvalTree
//             wraps), stencil base floor(xN)-1, indices taken mod N.
// The periodic step runs its stencil sums in double-float unless the
// context asks for FP64 sums (TBSLAS_SUMS_FP64); the free-space step is FP64
// (its interpolant jumps to 0 at the domain boundary, so a departure point
// must not move by a rounding).
#include "internal.h"

namespace tbg {

struct Stencil {
  int64_t ix[4], iy[4], iz[4];  // x offsets, y*N, z*N*N
  double wx[4], wy[4], wz[4];
};

// Builds the stencil of a point; returns false when the point evaluates to 0.
// Under PERIODIC the coordinates are wrapped in place.  nl >= 0 (periodic,
// N = 2^nl): stencil bases and offsets by grid_split_pow2, the same values
// without FP64 instructions.
__device__ __forceinline__ bool make_stencil(double& x, double& y, double& z, int N,
                                             bool periodic, Stencil& s, int nl = -1) {
  if (periodic) wrap3(x, y, z);
  if (!inside(x, y, z, periodic)) return false;
  const double scale = periodic ? (double)N : (double)(N - 1);
  const double c[3] = {x, y, z};
  int64_t base[3];
  double t[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    if (periodic && nl >= 0) {
      int g;
      grid_split_pow2(c[j], nl, g, t[j]);
      base[j] = g;
      continue;
    }
    const double p = c[j] * scale;
    int64_t g = (int64_t)p - 1;
    if (!periodic) {
      if (g < 0) g = 0;
      if (g > N - 4) g = N - 4;
    }
    base[j] = g;
    t[j] = p - (double)g;
  }
  if (periodic && nl >= 0) {
    lagrange4_unit(t[0], s.wx);
    lagrange4_unit(t[1], s.wy);
    lagrange4_unit(t[2], s.wz);
  } else {
    lagrange4(t[0], s.wx);
    lagrange4(t[1], s.wy);
    lagrange4(t[2], s.wz);
  }
  const int64_t NN = (int64_t)N * N;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int64_t gx = base[0] + k, gy = base[1] + k, gz = base[2] + k;
    if (periodic) {
      gx = gx < 0 ? gx + N : (gx >= N ? gx - N : gx);
      gy = gy < 0 ? gy + N : (gy >= N ? gy - N : gy);
      gz = gz < 0 ? gz + N : (gz >= N ? gz - N : gz);
    }
    s.ix[k] = gx;
    s.iy[k] = gy * N;
    s.iz[k] = gz * NN;
  }
  return true;
}

// sum_{j2} wz sum_{j1} wy sum_{j0} wx v : separable form of the reference's
// 64-term sum (same terms, grouped per axis).  The z planes stay a rolled
// loop: with 16 loads in flight instead of 64 the FP64 step fits 128
// registers and two CTAs per SM (the FP64 pipe stays fed; the arithmetic
// and its order are unchanged).
__device__ __forceinline__ double apply_stencil(const double* __restrict__ g, const Stencil& s) {
  double u = 0.0;
#pragma unroll 1
  for (int j2 = 0; j2 < 4; ++j2) {
    // the plane's offset and weight by selects, not by a run-time index:
    // the stencil then stays in registers instead of local memory
    const int64_t iz = j2 == 0 ? s.iz[0] : (j2 == 1 ? s.iz[1] : (j2 == 2 ? s.iz[2] : s.iz[3]));
    const double wz = j2 == 0 ? s.wz[0] : (j2 == 1 ? s.wz[1] : (j2 == 2 ? s.wz[2] : s.wz[3]));
    double v = 0.0;
#pragma unroll
    for (int j1 = 0; j1 < 4; ++j1) {
      const double* row = g + iz + s.iy[j1];
      double w = 0.0;
#pragma unroll
      for (int j0 = 0; j0 < 4; ++j0) w = fma(s.wx[j0], __ldg(row + s.ix[j0]), w);
      v = fma(s.wy[j1], w, v);
    }
    u = fma(wz, v, u);
  }
  return u;
}

__global__ void __launch_bounds__(256) k_fast_interp(const double* __restrict__ grid, int dof,
                                                     int N, const double* __restrict__ pts,
                                                     int64_t n, double* __restrict__ out,
                                                     int periodic) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
  Stencil s;
  const int64_t N3 = (int64_t)N * N * N;
  if (!make_stencil(x, y, z, N, periodic != 0, s)) {
    for (int k = 0; k < dof; ++k) out[i * dof + k] = 0.0;
    return;
  }
  for (int k = 0; k < dof; ++k) out[i * dof + k] = apply_stencil(grid + k * N3, s);
}

// Fused grid SL step, one thread per node (x fastest: coalesced node reads
// and output writes).  On a periodic power-of-two grid the first velocity
// evaluation of the first sub-step sits exactly on the node (the Lagrange
// weights there are exactly 0,1,0,0), so it is read, not interpolated.
// h = the node spacing and half_tau = tau / 2, formed once on the host.
__global__ void __launch_bounds__(256, 2) k_semilag_grid(const double* __restrict__ vel,
                                                      const double* __restrict__ con,
                                                      double* __restrict__ cout, int N,
                                                      double tau, double half_tau, double h,
                                                      int nrk, int periodic, int nl) {
  const bool node_read = nl >= 0;  // periodic power-of-two grid
  const int64_t N3 = (int64_t)N * N * N;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= N3) return;
  const bool per = periodic != 0;
  int64_t ix, iy, iz;
  if (nl >= 0) {  // N = 2^nl: the node's indices by shifts (no 64-bit division)
    ix = t & (N - 1);
    iy = (t >> nl) & (N - 1);
    iz = t >> (2 * nl);
  } else {
    ix = t % N;
    iy = (t / N) % N;
    iz = t / ((int64_t)N * N);
  }
  double x, y, z;
  if (nl >= 0) {
    x = grid_coord_pow2(ix, nl);
    y = grid_coord_pow2(iy, nl);
    z = grid_coord_pow2(iz, nl);
  } else {
    x = (double)ix * h;
    y = (double)iy * h;
    z = (double)iz * h;
  }
  double px = x, py = y, pz = z;
#pragma unroll 1
  for (int st = 0; st < 2 * nrk; ++st) {
    double v[3];
    if (st == 0 && node_read) {
      v[0] = __ldg(vel + t);
      v[1] = __ldg(vel + N3 + t);
      v[2] = __ldg(vel + 2 * N3 + t);
    } else {
      Stencil s;
      if (make_stencil(px, py, pz, N, per, s, nl)) {
        v[0] = apply_stencil(vel, s);
        v[1] = apply_stencil(vel + N3, s);
        v[2] = apply_stencil(vel + 2 * N3, s);
      } else {
        v[0] = v[1] = v[2] = 0.0;
      }
    }
    if ((st & 1) == 0) {
      x = px;
      y = py;
      z = pz;
      px = x + half_tau * v[0];
      py = y + half_tau * v[1];
      pz = z + half_tau * v[2];
    } else {
      x = x + tau * v[0];
      y = y + tau * v[1];
      z = z + tau * v[2];
      px = x;
      py = y;
      pz = z;
    }
  }
  Stencil s;
  cout[t] = make_stencil(x, y, z, N, per, s, nl) ? apply_stencil(con, s) : 0.0;
}

// Stencil of the double-float path: grid indices per axis (32-bit; the
// addresses are formed per row), weights in double-float.
struct StencilDF {
  int gx[4], gy[4], gz[4];
};

// Double-float form of apply_stencil: the same 64 terms and grouping, the
// sums on the FP32 pipe (df64.cuh) over a hi/lo split copy of the grid.
__device__ __forceinline__ df apply_stencil_df(const float2* __restrict__ g, const StencilDF& s,
                                               int N, const df (&wx)[4], const df (&wy)[4],
                                               const df (&wz)[4]) {
  const int64_t NN = (int64_t)N * N;
  df u{0.f, 0.f};
#pragma unroll 1
  for (int j2 = 0; j2 < 4; ++j2) {
    df v{0.f, 0.f};
#pragma unroll
    for (int j1 = 0; j1 < 4; ++j1) {
      const float2* row = g + (int64_t)s.gz[j2] * NN + (int64_t)s.gy[j1] * N;
      df w{0.f, 0.f};
#pragma unroll
      for (int j0 = 0; j0 < 4; ++j0) {
        const float2 c = __ldg(row + s.gx[j0]);
        df_fma_acc(w, df{c.x, c.y}, wx[j0]);
      }
      df_fma_acc(v, wy[j1], df_norm(w));
    }
    df_fma_acc(u, wz[j2], df_norm(v));
  }
  return df_norm(u);
}

// a - l for a small integer l, as an unnormalised double-float (TwoSum of
// the high word, exact)
__device__ __forceinline__ df df_sub_small(df a, float l) {
  const float s = __fsub_rn(a.hi, l);
  const float v = __fsub_rn(s, a.hi);
  const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(-l, v));
  return df{s, __fadd_rn(err, a.lo)};
}

__device__ __forceinline__ df df_mul_n(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df{p, e};
}

// The four cubic Lagrange weights at offset t (the products of lagrange4) in
// double-float, from the hi/lo split of the FP64 offset: ~25 FP32
// instructions a weight instead of FP64 products (relative error ~2^-46).
__device__ __forceinline__ void lagrange4_df(double t, df (&w)[4]) {
  const df td = df_split_bits(t);
  const df d0 = td, d1 = df_sub_small(td, 1.f), d2 = df_sub_small(td, 2.f),
           d3 = df_sub_small(td, 3.f);
  // den = -1/6, 1/2, -1/2, 1/6; 1/6 as a hi/lo pair
  const df sixth{0x1.555556p-3f, -0x1.555556p-28f};
  const df m6{-sixth.hi, -sixth.lo};
  w[0] = df_norm(df_mul_n(df_mul_n(df_mul_n(m6, d1), d2), d3));
  w[1] = df_norm(df_mul_n(df_mul_n(df_mul_n(df{0.5f, 0.f}, d0), d2), d3));
  w[2] = df_norm(df_mul_n(df_mul_n(df_mul_n(df{-0.5f, 0.f}, d0), d1), d3));
  w[3] = df_norm(df_mul_n(df_mul_n(df_mul_n(sixth, d0), d1), d2));
}


// Stencil of a point on the periodic grid for the double-float sums: the
// indices of make_stencil, the weights from lagrange4_df.  Returns false for
// a coordinate that is not a number (the FP64 path's "outside": value 0).
// nl >= 0: N = 2^nl (integer stencil bases), else FP64 bases.
__device__ __forceinline__ bool make_stencil_df(double& x, double& y, double& z, int N, int nl,
                                                StencilDF& s, df (&wx)[4], df (&wy)[4],
                                                df (&wz)[4]) {
  wrap3(x, y, z);
  if (!inside(x, y, z, true)) return false;
  const double c[3] = {x, y, z};
  int base[3];
  double t[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    if (nl >= 0) {
      grid_split_pow2(c[j], nl, base[j], t[j]);
    } else {
      const double p = c[j] * (double)N;
      const int64_t g = (int64_t)p - 1;
      base[j] = (int)g;
      t[j] = p - (double)g;
    }
  }
  lagrange4_df(t[0], wx);
  lagrange4_df(t[1], wy);
  lagrange4_df(t[2], wz);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int gx = base[0] + k, gy = base[1] + k, gz = base[2] + k;
    gx = gx < 0 ? gx + N : (gx >= N ? gx - N : gx);
    gy = gy < 0 ? gy + N : (gy >= N ? gy - N : gy);
    gz = gz < 0 ? gz + N : (gz >= N ? gz - N : gz);
    s.gx[k] = gx;
    s.gy[k] = gy;
    s.gz[k] = gz;
  }
  return true;
}

// The periodic grid step with the stencil sums in double-float: coordinates,
// stencil bases, the offsets t and the RK2 updates stay FP64; the Lagrange
// weights are formed from t in double-float.  The
// periodic tricubic interpolant is continuous everywhere, so the ~1e-17
// difference of a departure point from the FP64 one cannot move a value by
// more than the sums' own rounding (~1e-14 relative).  vel2/con2: hi/lo
// copies of the FP64 grids.
__global__ void __launch_bounds__(256, 4) k_semilag_grid_df(const double* __restrict__ vel,
                                                         const float2* __restrict__ vel2,
                                                         const float2* __restrict__ con2,
                                                         double* __restrict__ cout, int N,
                                                         double tau, int nrk, int nl) {
  const int node_read = nl >= 0;  // power-of-two grid: the first stage sits on the node
  const int64_t N3 = (int64_t)N * N * N;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= N3) return;
  const double h = 1.0 / N;
  const int64_t ix = t % N, iy = (t / N) % N, iz = t / ((int64_t)N * N);
  double x = (double)ix * h, y = (double)iy * h, z = (double)iz * h;
  const double half_tau = 0.5 * tau;
  double px = x, py = y, pz = z;
#pragma unroll 1
  for (int st = 0; st < 2 * nrk; ++st) {
    double v[3];
    if (st == 0 && node_read) {
      v[0] = __ldg(vel + t);
      v[1] = __ldg(vel + N3 + t);
      v[2] = __ldg(vel + 2 * N3 + t);
    } else {
      StencilDF s;
      df wx[4], wy[4], wz[4];
      if (make_stencil_df(px, py, pz, N, nl, s, wx, wy, wz)) {
        v[0] = df_to_double(apply_stencil_df(vel2, s, N, wx, wy, wz));
        v[1] = df_to_double(apply_stencil_df(vel2 + N3, s, N, wx, wy, wz));
        v[2] = df_to_double(apply_stencil_df(vel2 + 2 * N3, s, N, wx, wy, wz));
      } else {
        v[0] = v[1] = v[2] = 0.0;
      }
    }
    if ((st & 1) == 0) {
      x = px;
      y = py;
      z = pz;
      px = x + half_tau * v[0];
      py = y + half_tau * v[1];
      pz = z + half_tau * v[2];
    } else {
      x = x + tau * v[0];
      y = y + tau * v[1];
      z = z + tau * v[2];
      px = x;
      py = y;
      pz = z;
    }
  }
  StencilDF s;
  df wx[4], wy[4], wz[4];
  cout[t] = make_stencil_df(x, y, z, N, nl, s, wx, wy, wz)
                ? df_to_double(apply_stencil_df(con2, s, N, wx, wy, wz))
                : 0.0;
}

// hi/lo split of an FP64 grid (integer operations), flagging values outside
// the double-float range.
__global__ void k_split_grid(const double* __restrict__ g, float2* __restrict__ g2, int64_t n,
                             uint32_t* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = g[i];
    check_df_range(x, err);
    const df v = df_split_bits(x);
    g2[i] = make_float2(v.hi, v.lo);
  }
}

void launch_fast_interp(const double* grid, int dof, int nreg, const double* pts, int64_t n,
                        double* out, int periodic, cudaStream_t s) {
  if (n <= 0) return;
  k_fast_interp<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(grid, dof, nreg, pts, n, out,
                                                            periodic);
}

void launch_semilag_grid(const double* vel, const double* con, double* cout, int nreg,
                         double tau, int nrk, int periodic, cudaStream_t s) {
  const int64_t n = (int64_t)nreg * nreg * nreg;
  const bool pow2 = (nreg & (nreg - 1)) == 0;
  int nl = -1;
  if (periodic && pow2)
    for (nl = 0; (1 << nl) < nreg; ++nl) {
    }
  const double h = periodic ? 1.0 / nreg : 1.0 / (nreg - 1);
  k_semilag_grid<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(vel, con, cout, nreg, tau,
                                                             0.5 * tau, h, nrk, periodic, nl);
}

void launch_semilag_grid_df(const double* vel, const double* con, double* cout, int nreg,
                            double tau, int nrk, float2* vel2, float2* con2, uint32_t* err,
                            int num_sms, bool split_vel, cudaStream_t s) {
  const int64_t n = (int64_t)nreg * nreg * nreg;
  const bool pow2 = (nreg & (nreg - 1)) == 0;
  const int split_grid = num_sms * 8;
  if (split_vel) k_split_grid<<<split_grid, 256, 0, s>>>(vel, vel2, 3 * n, err);
  k_split_grid<<<split_grid, 256, 0, s>>>(con, con2, n, err);
  int nl = -1;
  if (pow2)
    for (nl = 0; (1 << nl) < nreg; ++nl) {
    }
  k_semilag_grid_df<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(vel, vel2, con2, cout, nreg, tau,
                                                                nrk, nl);
}

}  // namespace tbg
