// Templated tree kernels of the SL path, instantiated per Chebyshev degree by
// the tree_deg_*.cu translation units.
#pragma once

#include "internal.h"

namespace tbg {

// ---------------------------------------------------------------------------
// mbarrier + bulk-copy (TMA) helpers, inline PTX (sm_90+ forms).
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit` polls (each try_wait itself blocks for
// a hardware-defined time slice), so a lost transaction cannot hang the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// 1-D bulk copy global -> shared, completion signalled on `bar`.  src, dst
// 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// nrk midpoint-RK2 sub-steps of (x,y,z) through the velocity tree:
//   V = v(X); X* = X + tau/2 V; V = v(X*); X = X + tau V
// (IntegrateRK2 / ComputeTrajRK2, src/semilag/traj.inc:20-68).  The first
// evaluation of each sub-step wraps X in place under periodic boundaries and
// the update uses the wrapped X, as the reference's aliasing of xinit and
// xsol does.  One evaluation site serves both stages (smaller code).  The
// updates are fused multiply-adds, matching the oracle operation for
// operation, so departure points are bit-identical to it.
template <int D>
__device__ __forceinline__ void rk2_backtrace(const TreeView& vel, double& x, double& y,
                                              double& z, double tau, int nrk, bool per) {
  const double half_tau = 0.5 * tau;
  double px = x, py = y, pz = z;
#pragma unroll 1
  for (int st = 0; st < 2 * nrk; ++st) {
    double v[3];
    eval_point<D, 3>(vel, px, py, pz, per, v);
    if ((st & 1) == 0) {
      x = px;
      y = py;
      z = pz;
      px = fma(half_tau, v[0], x);
      py = fma(half_tau, v[1], y);
      pz = fma(half_tau, v[2], z);
    } else {
      x = fma(tau, v[0], x);
      y = fma(tau, v[1], y);
      z = fma(tau, v[2], z);
      px = x;
      py = y;
      pz = z;
    }
  }
}

// rk2_backtrace of a target node whose first-stage velocity vn (3 values) is
// known -- the node-grid evaluation, bit-identical to eval_point at X: X is
// wrapped in place as eval_point would, then the sub-steps continue as
// rk2_backtrace.  mid (or null) receives the first sub-step's midpoint.
template <int D>
__device__ __forceinline__ void rk2_backtrace_from_node(const TreeView& vel, const double* vn,
                                                        double& x, double& y, double& z,
                                                        double tau, int nrk, bool per,
                                                        double* mid = nullptr) {
  if (per) wrap3(x, y, z);
  const double half_tau = 0.5 * tau;
  double px = fma(half_tau, __ldg(vn + 0), x);
  double py = fma(half_tau, __ldg(vn + 1), y);
  double pz = fma(half_tau, __ldg(vn + 2), z);
  if (mid) {
    mid[0] = px;
    mid[1] = py;
    mid[2] = pz;
  }
  double v[3];
  eval_point<D, 3>(vel, px, py, pz, per, v);
  x = fma(tau, v[0], x);
  y = fma(tau, v[1], y);
  z = fma(tau, v[2], z);
  if (nrk > 1) rk2_backtrace<D>(vel, x, y, z, tau, nrk - 1, per);
}

// p[3t .. 3t+2] = (x, y, z) unless p is null.
__device__ __forceinline__ void store_point(double* p, int64_t t, double x, double y, double z) {
  if (p) {
    p[3 * t + 0] = x;
    p[3 * t + 1] = y;
    p[3 * t + 2] = z;
  }
}

// ---------------------------------------------------------------------------
// Fused in-situ SL step, one thread per target node of `con`:
//   target  = leaf anchor + 2^-depth * node           (tree_utils.h:484-491)
//   nrk x { V=v(X); X*=X+tau/2 V; V=v(X*); X=X+tau V } (traj.inc:20-68)
//   value   = c(X)                                     (semilag.inc:43)
// Targets and departure points never touch memory; only the node values are
// written, [leaf][node], for the refit.
// POINTS: only the midpoints and departure points (xmid, xdep required, vn
// given, nrk = 1) -- the adjoint's recomputation; no value is written.
template <int D, bool POINTS = false>
__global__ void __launch_bounds__(128) k_semilag_tree(const SemilagTreeArgs a) {
  constexpr int NP = D * D * D;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= a.con.L * NP) return;
  const int64_t leaf = t / NP;
  const int p = (int)(t - leaf * NP);
  const Geom g = load_geom(a.con.geom + leaf);
  const double h = leaf_side(g);  // 2^-depth, exact
  double x = g.x + h * a.nodes.x[p % D];
  double y = g.y + h * a.nodes.x[(p / D) % D];
  double z = g.z + h * a.nodes.x[p / (D * D)];
  const bool per = a.periodic != 0;
  if (a.vn)
    rk2_backtrace_from_node<D>(a.vel, a.vn + 3 * node_source(a.face, t), x, y, z, a.tau, a.nrk,
                               per, a.xmid ? a.xmid + 3 * t : nullptr);
  else
    rk2_backtrace<D>(a.vel, x, y, z, a.tau, a.nrk, per);
  store_point(a.xdep, t, x, y, z);
  if (POINTS) return;
  double c[1];
  eval_point<D, 1>(a.con, x, y, z, per, c);
  a.vals[t] = c[0];
}

template <int D>
void launch_semilag_tree(const SemilagTreeArgs& a, cudaStream_t s) {
  constexpr int NP = D * D * D;
  const int64_t n = a.con.L * NP;
  const int threads = 128;
  const int64_t blocks = (n + threads - 1) / threads;
  if (blocks > 0) k_semilag_tree<D><<<(unsigned)blocks, threads, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// The fused step with the Chebyshev sums in double-float (df64.cuh) and
// everything else -- targets, T_k recurrences, RK2 updates, Morton keys, leaf
// search, local coordinates -- in FP64.  Each coordinate carries a bound on
// its distance from the all-FP64 coordinate (eval_point_df / df_update); a
// target whose midpoint or departure point falls within that bound of a face
// of its leaf is appended to fix_list and recomputed by k_semilag_fix with
// the FP64 kernel body, so every leaf choice is the FP64 path's.  Values
// differ from the FP64 path by the sums' rounding (~1e-14).
// Seven (degree > 9) or eight 128-thread CTAs per SM (<= 72 / 64
// registers): the row loads of the sums wait on L1, and 28-32 resident warps
// hide that better than 16 warps without spills (measured on GB300: q = 14
// 309 -> 354 M points/s, q = 8 787 -> 879 M; five CTAs per SM was slower
// than four).
// POINTS: only the midpoints and departure points (xmid, xdep required,
// nrk = 1) -- the departure point's lookup in con is checked for ambiguity
// but not summed, and no value is written.
template <int D, bool POINTS = false>
__global__ void __launch_bounds__(128, (D <= 10 ? 8 : 7)) k_semilag_tree_df(const SemilagTreeArgs a) {
  constexpr int NP = D * D * D;
  extern __shared__ float2 s_slots[];
  const ThreadSlots slots{s_slots + threadIdx.x, (int)blockDim.x};
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= a.con.L * NP) return;
  const int64_t leaf = t / NP;
  const int p = (int)(t - leaf * NP);
  const Geom g = load_geom(a.con.geom + leaf);
  const double h = leaf_side(g);
  double x[3] = {g.x + h * a.nodes.x[p % D], g.y + h * a.nodes.x[(p / D) % D],
                 g.z + h * a.nodes.x[p / (D * D)]};
  const bool per = a.periodic != 0;
  const double half_tau = 0.5 * a.tau;
  double px[3] = {x[0], x[1], x[2]};
  double m0[3] = {0.0, 0.0, 0.0}, mp[3] = {0.0, 0.0, 0.0};
  bool amb = false;
  int st0 = 0;
  if (a.vn) {
    // first stage from the velocity at the nodes, bit-identical to the FP64
    // path's v(X): X wrapped in place as eval_point does, the midpoint exact
    const double* vn = a.vn + 3 * node_source(a.face, t);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (per) x[k] = wrap1(x[k]);
      px[k] = fma(half_tau, __ldg(vn + k), x[k]);
    }
    st0 = 1;
    store_point(a.xmid, t, px[0], px[1], px[2]);
  }
#pragma unroll 1
  for (int st = st0; st < 2 * a.nrk; ++st) {
    double v[3], ev[3];
    amb |= eval_point_df<D, 3, true>(a.vel, px[0], px[1], px[2], per, mp, v, ev, slots);
    if ((st & 1) == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = px[k];
        df_update(half_tau, v[k], ev[k], x[k], m0[k], px[k], mp[k]);
      }
      store_point(a.xmid, t, px[0], px[1], px[2]);
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        df_update(a.tau, v[k], ev[k], x[k], m0[k], x[k], m0[k]);
        px[k] = x[k];
        mp[k] = m0[k];
      }
    }
  }
  store_point(a.xdep, t, x[0], x[1], x[2]);
  if (POINTS) {
    amb |= lookup_ambiguous(a.con, x[0], x[1], x[2], per, m0);
  } else {
    double c[1], ce[1];
    amb |= eval_point_df<D, 1, false>(a.con, x[0], x[1], x[2], per, m0, c, ce, slots);
    a.vals[t] = c[0];
  }
  if (amb) a.fix_list[atomicAdd(a.fix_count, 1ull)] = t;
}

// FP64 recomputation of the listed targets (the arithmetic of
// k_semilag_tree, with the first-stage velocity from the node grid when
// given -- it is bit-identical to eval_point there); stored midpoints and
// departure points of those targets become the FP64 path's.
template <int D, bool POINTS = false>
__global__ void __launch_bounds__(128) k_semilag_fix(const SemilagTreeArgs a) {
  constexpr int NP = D * D * D;
  const int64_t n = (int64_t)*a.fix_count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = a.fix_list[i];
    const int64_t leaf = t / NP;
    const int p = (int)(t - leaf * NP);
    const Geom g = load_geom(a.con.geom + leaf);
    const double h = leaf_side(g);
    double x = g.x + h * a.nodes.x[p % D];
    double y = g.y + h * a.nodes.x[(p / D) % D];
    double z = g.z + h * a.nodes.x[p / (D * D)];
    const bool per = a.periodic != 0;
    if (a.vn)
      rk2_backtrace_from_node<D>(a.vel, a.vn + 3 * node_source(a.face, t), x, y, z, a.tau,
                                 a.nrk, per, a.xmid ? a.xmid + 3 * t : nullptr);
    else
      rk2_backtrace<D>(a.vel, x, y, z, a.tau, a.nrk, per);
    store_point(a.xdep, t, x, y, z);
    if (!POINTS) {
      double c[1];
      eval_point<D, 1>(a.con, x, y, z, per, c);
      a.vals[t] = c[0];
    }
  }
}

template <int D>
void launch_semilag_tree_df(const SemilagTreeArgs& a, cudaStream_t s) {
  constexpr int NP = D * D * D;
  const int64_t n = a.con.L * NP;
  const int threads = 128;
  const int64_t blocks = (n + threads - 1) / threads;
  if (blocks == 0) return;
  cudaMemsetAsync(a.fix_count, 0, sizeof(unsigned long long), s);
  const size_t smem = 2 * D * threads * sizeof(float2);
  k_semilag_tree_df<D><<<(unsigned)blocks, threads, smem, s>>>(a);
  k_semilag_fix<D><<<a.fix_grid, threads, 0, s>>>(a);
}

// Midpoints and departure points only, FP64 (the FP64 adjoint's recompute).
template <int D>
void launch_points_fp64(const SemilagTreeArgs& a, cudaStream_t s) {
  constexpr int NP = D * D * D;
  const int64_t n = a.con.L * NP;
  const int threads = 128;
  const int64_t blocks = (n + threads - 1) / threads;
  if (blocks > 0) k_semilag_tree<D, true><<<(unsigned)blocks, threads, 0, s>>>(a);
}

// Midpoints and departure points only (the double-float adjoint's recompute).
template <int D>
void launch_points_df(const SemilagTreeArgs& a, cudaStream_t s) {
  constexpr int NP = D * D * D;
  const int64_t n = a.con.L * NP;
  const int threads = 128;
  const int64_t blocks = (n + threads - 1) / threads;
  if (blocks == 0) return;
  cudaMemsetAsync(a.fix_count, 0, sizeof(unsigned long long), s);
  const size_t smem = 2 * D * threads * sizeof(float2);
  k_semilag_tree_df<D, true><<<(unsigned)blocks, threads, smem, s>>>(a);
  k_semilag_fix<D, true><<<a.fix_grid, threads, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// RK2 backtrace of arbitrary points (ComputeTrajRK2, traj.inc:48-68), one
// thread per point, direct leaf lookup per stage.
template <int D>
__global__ void __launch_bounds__(128) k_traj(const TrajArgs a) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double x = a.x[3 * i + 0], y = a.x[3 * i + 1], z = a.x[3 * i + 2];
  rk2_backtrace<D>(a.vel, x, y, z, a.tau, a.nrk, a.periodic != 0);
  a.xdep[3 * i + 0] = x;
  a.xdep[3 * i + 1] = y;
  a.xdep[3 * i + 2] = z;
}

template <int D>
void launch_traj(const TrajArgs& a, cudaStream_t s) {
  const int threads = 128;
  const int64_t blocks = (a.n + threads - 1) / threads;
  if (blocks > 0) k_traj<D><<<(unsigned)blocks, threads, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// Leaf-staged evaluation of bucketed points (EvalNodesLocal,
// tree_functor.h:155-395).  Persistent CTAs walk the tile list; per tile the
// leaf's coefficient block is bulk-copied (TMA) into shared memory while the
// threads load their point and build T_k(x), T_j(y), T_i(z); then every
// thread sums from shared memory (warp-uniform addresses: broadcasts).
template <int D>
__global__ void __launch_bounds__(kTile) k_eval_tiles(const EvalTilesArgs a) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  extern __shared__ __align__(16) double s_coeff[];
  __shared__ __align__(8) uint64_t bar;
  const TreeView& t = a.tree;
  const int64_t ntiles = *a.ntiles;
  const uint32_t bytes = (uint32_t)(t.stride * sizeof(double));
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  uint32_t parity = 0;
  const bool per = a.periodic != 0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const Tile tl = a.tiles[tile];
    if (threadIdx.x == 0) {
      fence_proxy_async_smem();
      mbar_expect_tx(&bar, bytes);
      bulk_g2s(s_coeff, t.coeff + (int64_t)tl.leaf * t.stride, bytes, &bar);
    }
    const bool active = threadIdx.x < tl.count;
    int64_t i = 0;
    double tx[D], ty[D], tz[D];
    if (active) {
      i = a.perm[tl.start + threadIdx.x];
      double x = a.pos[3 * i + 0], y = a.pos[3 * i + 1], z = a.pos[3 * i + 2];
      if (per) {
        x = wrap1(x);
        y = wrap1(y);
        z = wrap1(z);
      }
      const Geom g = load_geom(t.geom + tl.leaf);
      cheb_T<D>((x - g.x) * g.w - 1.0, tx);
      cheb_T<D>((y - g.y) * g.w - 1.0, ty);
      cheb_T<D>((z - g.z) * g.w - 1.0, tz);
    }
    const bool timed_out = !mbar_wait_bounded(&bar, parity, a.wait_limit);
    parity ^= 1u;
    if (__syncthreads_or(timed_out)) {
      if (threadIdx.x == 0) {
        atomicOr(a.err, kErrBarrierTimeout);
        mbar_wait_bounded(&bar, parity ^ 1u, kWaitLimit);  // let the copy land
      }
      return;
    }
    if (active) {
      for (int l = 0; l < t.dof; ++l)
        a.out[i * t.dof + l] = tri_sum<D>(SharedLoad{s_coeff + l * NC}, tx, ty, tz);
    }
    __syncthreads();  // shared block free before the next copy
  }
}

template <int D>
void launch_eval_tiles(const EvalTilesArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)a.tree.stride * sizeof(double);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_eval_tiles<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    attr_set = true;
  }
  if (a.grid > 0) k_eval_tiles<D><<<a.grid, kTile, smem, s>>>(a);
}

template <int D>
void register_degree(DegreeKernels* table) {
  table[D - 1].semilag = &launch_semilag_tree<D>;
  table[D - 1].semilag_df = &launch_semilag_tree_df<D>;
  table[D - 1].traj = &launch_traj<D>;
  table[D - 1].eval_tiles = &launch_eval_tiles<D>;
  if constexpr (D <= 11) {  // the adjoint's degrees
    table[D - 1].points_df = &launch_points_df<D>;
    table[D - 1].points_fp64 = &launch_points_fp64<D>;
  }
}

}  // namespace tbg
