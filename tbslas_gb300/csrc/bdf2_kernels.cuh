// Second-order (BDF2) semi-Lagrangian step with two backtraces, instantiated
// per Chebyshev degree by bdf2_deg_*.cu.  The reference's advection-diffusion
// driver (src/applications/src/advdiff-ss.cpp:485-521) computes, for every
// Chebyshev node X of the merged tree treen,
//   X1 = ComputeTrajRK2(vel, X,  t, t - dt)       c_n    at X1 (tree treec)
//   X2 = ComputeTrajRK2(vel, X1, t - dt, t - 2dt) c_{n-1} at X2 (tree treep)
//   value = 4/3 c_n(X1) - 1/3 c_{n-1}(X2)
// and refits treen (SetTreeGridValues).  The second backtrace starts from X1
// as the concentration evaluation left it (wrapped in place under periodic
// boundaries, the aliasing of EvalTree's coordinate array).  One thread per
// target; the velocity at the targets (first stage) comes from the node grid.
#pragma once

#include "tree_kernels.cuh"

namespace tbg {

// 4/3 a - 1/3 b, the two products and the difference rounded separately (the
// reference's `ccoeff * c - pcoeff * p` without contraction).
__device__ __forceinline__ double bdf2_combine(double a, double b) {
  return __dsub_rn(__dmul_rn(4.0 / 3, a), __dmul_rn(1.0 / 3, b));
}

// The FP64 arithmetic of one target (the FP64 step and the near-face pass).
template <int D>
__device__ __forceinline__ double bdf2_target_fp64(const Bdf2Args& a, int64_t t) {
  constexpr int NP = D * D * D;
  const int64_t leaf = t / NP;
  const int p = (int)(t - leaf * NP);
  const Geom g = load_geom(a.next.geom + leaf);
  const double h = leaf_side(g);
  double x = g.x + h * a.nodes.x[p % D];
  double y = g.y + h * a.nodes.x[(p / D) % D];
  double z = g.z + h * a.nodes.x[p / (D * D)];
  const bool per = a.periodic != 0;
  rk2_backtrace_from_node<D>(a.vel, a.vn + 3 * node_source(a.face, t), x, y, z, a.tau1, a.nrk,
                             per);
  double cn[1], cp[1];
  eval_point<D, 1>(a.cur, x, y, z, per, cn);  // wraps X1 in place
  rk2_backtrace<D>(a.vel, x, y, z, a.tau2, a.nrk, per);
  eval_point<D, 1>(a.prev, x, y, z, per, cp);
  return bdf2_combine(cn[0], cp[0]);
}

template <int D>
__global__ void __launch_bounds__(128) k_semilag_bdf2(const Bdf2Args a) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= a.next.L * D * D * D) return;
  a.vals[t] = bdf2_target_fp64<D>(a, t);
}

// RK2 sub-steps from st0 of the double-float step (k_semilag_tree_df's stage
// loop): x / px the point and midpoint, m0 / mp their distance bounds from the
// FP64 path; returns true if a lookup was ambiguous.
template <int D>
__device__ __forceinline__ bool rk2_df_stages(const TreeView& vel, double (&x)[3],
                                              double (&px)[3], double (&m0)[3], double (&mp)[3],
                                              int st0, int nrk, double tau, bool per,
                                              ThreadSlots slots) {
  const double half_tau = 0.5 * tau;
  bool amb = false;
#pragma unroll 1
  for (int st = st0; st < 2 * nrk; ++st) {
    double v[3], ev[3];
    amb |= eval_point_df<D, 3, true>(vel, px[0], px[1], px[2], per, mp, v, ev, slots);
    if ((st & 1) == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = px[k];
        df_update(half_tau, v[k], ev[k], x[k], m0[k], px[k], mp[k]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        df_update(tau, v[k], ev[k], x[k], m0[k], x[k], m0[k]);
        px[k] = x[k];
        mp[k] = m0[k];
      }
    }
  }
  return amb;
}

// Double-float sums, FP64 coordinates and lookups (as k_semilag_tree_df);
// targets whose lookup the bounds make ambiguous go to the FP64 pass.  Eight
// (degree <= 9) or seven CTAs per SM, as the single-backtrace kernel: with
// the two backtraces in one loop the register cap costs a few spills but the
// extra warps hide the coefficient loads (q = 8 on GB300: six CTAs 5.47 ms,
// seven 5.21 ms, eight 5.02 ms per step).
template <int D>
__global__ void __launch_bounds__(128, (D <= 10 ? 8 : 7)) k_semilag_bdf2_df(const Bdf2Args a) {
  constexpr int NP = D * D * D;
  extern __shared__ float2 s_slots[];
  const ThreadSlots slots{s_slots + threadIdx.x, (int)blockDim.x};
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= a.next.L * NP) return;
  const int64_t leaf = t / NP;
  const int p = (int)(t - leaf * NP);
  const Geom g = load_geom(a.next.geom + leaf);
  const double h = leaf_side(g);
  double x[3] = {g.x + h * a.nodes.x[p % D], g.y + h * a.nodes.x[(p / D) % D],
                 g.z + h * a.nodes.x[p / (D * D)]};
  const bool per = a.periodic != 0;
  double px[3], m0[3] = {0.0, 0.0, 0.0}, mp[3] = {0.0, 0.0, 0.0};
  // first stage from the node grid (exact)
  const double* vn = a.vn + 3 * node_source(a.face, t);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (per) x[k] = wrap1(x[k]);
    px[k] = fma(0.5 * a.tau1, __ldg(vn + k), x[k]);
  }
  // the two backtraces share one copy of the stage loop and of the
  // evaluation (the instruction caches hold one): pass 0 continues from the
  // midpoint and evaluates c_n at X1, pass 1 starts from X1 (wrapped in place
  // by that evaluation) and evaluates c_{n-1} at X2
  bool amb = false;
  double cv[2], e[1];
#pragma unroll 1
  for (int pass = 0; pass < 2; ++pass) {
    amb |= rk2_df_stages<D>(a.vel, x, px, m0, mp, pass == 0 ? 1 : 0, a.nrk,
                            pass == 0 ? a.tau1 : a.tau2, per, slots);
    double c[1];
    amb |= eval_point_df<D, 1, false>(pass == 0 ? a.cur : a.prev, x[0], x[1], x[2], per, m0, c,
                                      e, slots);
    cv[pass] = c[0];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      px[k] = x[k];
      mp[k] = m0[k];
    }
  }
  const double cn[1] = {cv[0]}, cp[1] = {cv[1]};
  a.vals[t] = bdf2_combine(cn[0], cp[0]);
  if (amb) a.fix_list[atomicAdd(a.fix_count, 1ull)] = t;
}

template <int D>
__global__ void __launch_bounds__(128) k_semilag_bdf2_fix(const Bdf2Args a) {
  const int64_t n = (int64_t)*a.fix_count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = a.fix_list[i];
    a.vals[t] = bdf2_target_fp64<D>(a, t);
  }
}

template <int D>
void launch_semilag_bdf2(const Bdf2Args& a, bool df_sums, cudaStream_t s) {
  const int64_t n = a.next.L * D * D * D;
  const int threads = 128;
  const int64_t blocks = (n + threads - 1) / threads;
  if (blocks == 0) return;
  if (!df_sums) {
    k_semilag_bdf2<D><<<(unsigned)blocks, threads, 0, s>>>(a);
    return;
  }
  cudaMemsetAsync(a.fix_count, 0, sizeof(unsigned long long), s);
  k_semilag_bdf2_df<D><<<(unsigned)blocks, threads, 2 * D * threads * sizeof(float2), s>>>(a);
  k_semilag_bdf2_fix<D><<<a.fix_grid, threads, 0, s>>>(a);
}

}  // namespace tbg
