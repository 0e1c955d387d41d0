// The adjoint step of adjoint_kernels.cuh with its sums in double-float
// (df64.cuh): the two gradient sums (grad c^k at Xd, grad(g . v) at X*) and
// the two CTA-cooperative scatters at those points run as hi/lo float pairs
// on the FP32 pipe; point locations, T_k and dT_k recurrences, the weights
// and the global accumulation (FP64 atomics) stay FP64, and the third
// scatter (at the node X) is the transposed node-grid pass.  The points are
// the step's own (checkpointed by the forward, whose leaf choices are the
// FP64 step's, or recomputed in FP64), so results differ from the FP64
// adjoint by the sums' rounding (~1e-15 relative).
#pragma once

#include "adjoint_f64.cuh"

namespace tbg {

// Targets (threads) per CTA of the double-float adjoint: 192 gives every warp
// one coefficient per scatter pass at q = 8 (Nc = 165); with 128 threads two
// warps carried a second coefficient and set the pace (measured on GB300,
// q = 8: 36.0 -> 34.0 ms per 4-step adjoint pass of a 4096-leaf tree).
constexpr int kAdjDfThreads = 192;

// The gradient's coefficients: one component, or sum_a g_a c_a over the three
// velocity components.
struct GradOne {
  const float2* __restrict__ c;
  __device__ __forceinline__ df operator()(int i) const {
    const float2 v = __ldg(c + i);
    return df{v.x, v.y};
  }
};
struct GradW3 {
  const float2* __restrict__ c;
  int nc;
  df g0, g1, g2;
  __device__ __forceinline__ df operator()(int i) const {
    const float2 a = __ldg(c + i), b = __ldg(c + nc + i), e = __ldg(c + 2 * nc + i);
    df s{0.f, 0.f};
    df_fma_acc(s, g0, df{a.x, a.y});
    df_fma_acc(s, g1, df{b.x, b.y});
    df_fma_acc(s, g2, df{e.x, e.y});
    return df_norm(s);
  }
};

#define TBG_DF_GTERM(K)                                                          \
  case (K) + 1:                                                                  \
    if constexpr ((K) < D) {                                                     \
      const df ct = ld(idx + (K));                                               \
      df_fma_acc(w, ct, tx[(K) < D ? (K) : 0]);                                  \
      df_fma_acc(wd, ct, dx[(K) < D ? (K) : 0]);                                 \
    }                                                                            \
    [[fallthrough]];

// (d/dxi, d/deta, d/dzeta) of the triangular expansion, rows rolled as in
// tri_sum_df_rows.
template <int D, class Load>
__device__ __forceinline__ void tri_grad_df(Load ld, const df (&tx)[D], const df (&dx)[D],
                                            ThreadSlots s, double (&g)[3]) {
  static_assert(D >= 1 && D <= 17, "degree above 16");
  df gx{0.f, 0.f}, gy{0.f, 0.f}, gz{0.f, 0.f};
  int idx = 0;
#pragma unroll 1
  for (int i = 0; i < D; ++i) {
    df vx{0.f, 0.f}, vy{0.f, 0.f}, vz{0.f, 0.f};
#pragma unroll 1
    for (int j = 0; j < D - i; ++j) {
      const int n = D - i - j;
      df w{0.f, 0.f}, wd{0.f, 0.f};
      switch (n) {
        TBG_DF_GTERM(16)
        TBG_DF_GTERM(15)
        TBG_DF_GTERM(14)
        TBG_DF_GTERM(13)
        TBG_DF_GTERM(12)
        TBG_DF_GTERM(11)
        TBG_DF_GTERM(10)
        TBG_DF_GTERM(9)
        TBG_DF_GTERM(8)
        TBG_DF_GTERM(7)
        TBG_DF_GTERM(6)
        TBG_DF_GTERM(5)
        TBG_DF_GTERM(4)
        TBG_DF_GTERM(3)
        TBG_DF_GTERM(2)
        TBG_DF_GTERM(1)
        TBG_DF_GTERM(0)
        default:
          break;
      }
      idx += n;
      w = df_norm(w);
      wd = df_norm(wd);
      const df tyj = s.get(j), dyj = s.get(D + j);
      df_fma_acc(vx, tyj, wd);
      df_fma_acc(vy, dyj, w);
      df_fma_acc(vz, tyj, w);
    }
    const df tzi = s.get(2 * D + i), dzi = s.get(3 * D + i);
    df_fma_acc(gx, tzi, df_norm(vx));
    df_fma_acc(gy, tzi, df_norm(vy));
    df_fma_acc(gz, dzi, df_norm(vz));
  }
  g[0] = df_to_double(df_norm(gx));
  g[1] = df_to_double(df_norm(gy));
  g[2] = df_to_double(df_norm(gz));
}
#undef TBG_DF_GTERM

// T_k, dT_k of a local coordinate (FP64 recurrences, then hi/lo split): x in
// registers, y and z in the thread's slots.
template <int D>
__device__ __forceinline__ void grad_tables(const Geom& g, double x, double y, double z,
                                            df (&tx)[D], df (&dx)[D], ThreadSlots s) {
  double T[D], dT[D];
  cheb_TdT<D>((x - g.x) * g.w - 1.0, T, dT);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    tx[k] = df_split_bits(T[k]);
    dx[k] = df_split_bits(dT[k]);
  }
  cheb_TdT<D>((y - g.y) * g.w - 1.0, T, dT);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    s.put(k, df_split_bits(T[k]));
    s.put(D + k, df_split_bits(dT[k]));
  }
  cheb_TdT<D>((z - g.z) * g.w - 1.0, T, dT);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    s.put(2 * D + k, df_split_bits(T[k]));
    s.put(3 * D + k, df_split_bits(dT[k]));
  }
}

// exact product hi*hi split plus the cross terms (un-normalised, as
// df_fma_acc accepts it)
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df{p, e};
}

// Shared memory of the double-float adjoint.  Every thread owns NS slots of
// one double-float each (ThreadSlots: element e of thread t at
// slots[e * BS + t]); the stride BS is odd, so that a warp reading element
// e_lane of one point's column -- the scatters, one coefficient per lane --
// touches distinct banks for distinct e.  Slot map of a point:
//   [0, D)    T_j(y)
//   [D, 2D)   dT_j(y) for the gradient, then T_k(x) for the scatter
//   [2D, 3D)  T_i(z)
//   [3D, 4D)  dT_i(z) for the gradient, then the scatter's weights
template <int D>
struct AdjDfShared {
  static constexpr int BS = kAdjDfThreads + 1;
  static constexpr int NS = 4 * D > 3 * D + 3 ? 4 * D : 3 * D + 3;
  float2 slots[NS * BS];
  int leaf[kAdjDfThreads];            // scatter leaf of each point (-1: none / done)
  unsigned char list[kAdjDfThreads];  // points of the leaf in progress
  int wcount[kAdjDfThreads / 32];
  int cur;
};

template <int D>
constexpr size_t adj_df_smem() {
  return sizeof(AdjDfShared<D>);
}

// Slot offsets of T_i(z), T_j(y), T_k(x) for this thread's scatter
// coefficients n = tid + c * blockDim (triangular order; oz < 0: none).
template <int D, int PER>
__device__ __forceinline__ void scatter_offsets(int (&oz)[PER], int (&oy)[PER], int (&ox)[PER]) {
  constexpr int BS = AdjDfShared<D>::BS;
#pragma unroll
  for (int c = 0; c < PER; ++c) {
    const int n = threadIdx.x + c * kAdjDfThreads;
    int idx = 0;
    oz[c] = -1;
    oy[c] = ox[c] = 0;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D - i; ++j) {
        const int len = D - i - j;
        if (n >= idx && n < idx + len) {
          oz[c] = (2 * D + i) * BS;
          oy[c] = j * BS;
          ox[c] = (D + n - idx) * BS;
        }
        idx += len;
      }
  }
}

// out[leaf*stride + l*NC + n] += w[l] * phi_n(point) for every thread's point
// (lf < 0: none).  The point's T_j(y) and T_i(z) are in its slots (from
// grad_tables), T_k(x) in tx.  For each distinct leaf among the block's
// points, in order of first appearance, the points of that leaf are listed
// (ballot compaction, in thread order) and every thread sums its
// coefficients over the list, adding each to global memory with one FP64
// atomic.  All threads of the block call it; it ends after a barrier that
// every thread passes once it has finished reading the slots.
template <int D, int DOF, int PER>
__device__ __forceinline__ void scatter_df(AdjDfShared<D>& sm, double* __restrict__ out,
                                           int64_t stride, int64_t lf, const df (&tx)[D],
                                           const double (&w)[DOF], const int (&oz)[PER],
                                           const int (&oy)[PER], const int (&ox)[PER]) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  constexpr int BS = AdjDfShared<D>::BS;
  constexpr int NW = kAdjDfThreads / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (lf >= 0) {
    float2* const col = sm.slots + tid;
#pragma unroll
    for (int k = 0; k < D; ++k) col[(D + k) * BS] = make_float2(tx[k].hi, tx[k].lo);
#pragma unroll
    for (int l = 0; l < DOF; ++l) {
      const df v = df_from_double(w[l]);
      col[(3 * D + l) * BS] = make_float2(v.hi, v.lo);
    }
  }
  const int my_leaf = lf >= 0 ? (int)lf : -1;
  sm.leaf[tid] = my_leaf;
  bool pending = my_leaf >= 0;
  __syncthreads();
  for (;;) {
    if (warp == 0) {
      int first = -1;
#pragma unroll
      for (int chunk = 0; chunk < NW; ++chunk) {
        const int v = sm.leaf[chunk * 32 + lane];
        const unsigned m = __ballot_sync(0xffffffffu, v >= 0);
        if (m) {
          first = __shfl_sync(0xffffffffu, v, __ffs(m) - 1);
          break;
        }
      }
      if (lane == 0) sm.cur = first;
    }
    __syncthreads();
    const int cur = sm.cur;
    if (cur < 0) break;
    const bool mine = pending && my_leaf == cur;
    const unsigned m = __ballot_sync(0xffffffffu, mine);
    if (lane == 0) sm.wcount[warp] = __popc(m);
    __syncthreads();
    int base = 0, total = 0;
#pragma unroll
    for (int w2 = 0; w2 < NW; ++w2) {
      const int c = sm.wcount[w2];
      base += w2 < warp ? c : 0;
      total += c;
    }
    if (mine) {
      sm.list[base + __popc(m & ((1u << lane) - 1u))] = (unsigned char)tid;
      sm.leaf[tid] = -1;
      pending = false;
    }
    __syncthreads();
    df acc[PER][DOF];
#pragma unroll
    for (int c = 0; c < PER; ++c)
#pragma unroll
      for (int l = 0; l < DOF; ++l) acc[c][l] = df{0.f, 0.f};
    for (int k = 0; k < total; ++k) {
      const float2* const pc = sm.slots + sm.list[k];
      df wp[DOF];
#pragma unroll
      for (int l = 0; l < DOF; ++l) {
        const float2 v = pc[(3 * D + l) * BS];
        wp[l] = df{v.x, v.y};
      }
#pragma unroll
      for (int c = 0; c < PER; ++c) {
        if (oz[c] < 0) continue;
        const float2 a = pc[oz[c]], b = pc[oy[c]], e = pc[ox[c]];
        const df t = df_mul(df_mul(df{a.x, a.y}, df{b.x, b.y}), df{e.x, e.y});
#pragma unroll
        for (int l = 0; l < DOF; ++l) df_fma_acc(acc[c][l], wp[l], t);
      }
    }
#pragma unroll
    for (int c = 0; c < PER; ++c) {
      if (oz[c] < 0) continue;
      const int n = tid + c * kAdjDfThreads;
#pragma unroll
      for (int l = 0; l < DOF; ++l) {
        const double v = df_to_double(df_norm(acc[c][l]));
        if (v != 0.0) atomicAdd(out + (int64_t)cur * stride + l * NC + n, v);
      }
    }
  }
}

// One thread per target node, its X* and Xd from a.xmid / a.xdep (required:
// the forward's checkpoints or the recompute's).  The tau^2/2 J_v(X*)^T g (x)
// phi(X) term goes to a.wnode (required) for the node-grid scatter.  Four
// (q <= 8) or three CTAs per SM.
template <int D>
__global__ void __launch_bounds__(kAdjDfThreads, (D <= 9 ? 4 : 3)) k_adjoint_df(const AdjArgs a,
                                                            const float2* __restrict__ con2) {
  constexpr int NP = D * D * D;
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  constexpr int PER = (NC + kAdjDfThreads - 1) / kAdjDfThreads;
  extern __shared__ __align__(16) unsigned char adj_df_raw[];
  AdjDfShared<D>& sm = *reinterpret_cast<AdjDfShared<D>*>(adj_df_raw);
  const ThreadSlots slots{sm.slots + threadIdx.x, AdjDfShared<D>::BS};
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < a.con.L * NP;
  const bool per = a.periodic != 0;
  const int64_t tt = active ? t : 0;
  double xs = a.xmid[3 * tt], ys = a.xmid[3 * tt + 1], zs = a.xmid[3 * tt + 2];
  double xd = a.xdep[3 * tt], yd = a.xdep[3 * tt + 1], zd = a.xdep[3 * tt + 2];
  const double mu = active ? a.mu[tt] : 0.0;
  int oz[PER], oy[PER], ox[PER];
  scatter_offsets<D, PER>(oz, oy, ox);

  // g = mu grad c^k(Xd); lambda^k += mu phi(Xd)
  double gvec[3] = {0.0, 0.0, 0.0};
  {
    Geom g;
    int64_t lf = locate<D>(a.con, xd, yd, zd, per, g);
    if (!active) lf = -1;
    df tx[D];
    if (lf >= 0) {
      df dx[D];
      grad_tables<D>(g, xd, yd, zd, tx, dx, slots);
      double gr[3];
      tri_grad_df<D>(GradOne{con2 + lf * NC}, tx, dx, slots, gr);
      gvec[0] = mu * gr[0] * g.w;
      gvec[1] = mu * gr[1] * g.w;
      gvec[2] = mu * gr[2] * g.w;
    }
    const double w[1] = {mu};
    scatter_df<D, 1, PER>(sm, a.lambda, NC, lf, tx, w, oz, oy, ox);
  }
  // tau g (x) phi(X*) and J_v(X*)^T g = grad(g . v)(X*)
  double jtg[3] = {0.0, 0.0, 0.0};
  {
    Geom g;
    int64_t lf = locate<D>(a.vel, xs, ys, zs, per, g);
    if (!active) lf = -1;
    df tx[D];
    if (lf >= 0) {
      df dx[D];
      grad_tables<D>(g, xs, ys, zs, tx, dx, slots);
      double gr[3];
      tri_grad_df<D>(GradW3{a.vel.coeff2 + lf * a.vel.stride, NC, df_from_double(gvec[0]),
                            df_from_double(gvec[1]), df_from_double(gvec[2])},
                     tx, dx, slots, gr);
      jtg[0] = gr[0] * g.w;
      jtg[1] = gr[1] * g.w;
      jtg[2] = gr[2] * g.w;
    }
    const double w[3] = {a.tau * gvec[0], a.tau * gvec[1], a.tau * gvec[2]};
    scatter_df<D, 3, PER>(sm, a.grad_vel, 3 * NC, lf, tx, w, oz, oy, ox);
  }
  // tau^2/2 J_v(X*)^T g (x) phi(X): X is a node, the node-grid scatter adds it
  if (active) {
    const double c2 = 0.5 * a.tau * a.tau;
    double* w = a.wnode + 3 * t;
    if (a.wnode_add) {
      w[0] += c2 * jtg[0];
      w[1] += c2 * jtg[1];
      w[2] += c2 * jtg[2];
    } else {
      w[0] = c2 * jtg[0];
      w[1] = c2 * jtg[1];
      w[2] = c2 * jtg[2];
    }
  }
}

template <int D>
void launch_adjoint_df(const AdjArgs& a, const float2* con2, cudaStream_t s) {
  const int64_t n = a.con.L * D * D * D;
  const size_t smem = adj_df_smem<D>();
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_adjoint_df<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  if (n > 0)
    k_adjoint_df<D><<<(unsigned)((n + kAdjDfThreads - 1) / kAdjDfThreads), kAdjDfThreads, smem, s>>>(
        a, con2);
}

template <int D>
void register_adjoint_degree(AdjFn* a, AdjDfFn* d, JacStepFn* j) {
  a[D - 1] = &launch_adjoint_f64<D>;
  d[D - 1] = &launch_adjoint_df<D>;
  j[D - 1] = &launch_semilag_tree_jac<D>;
}

}  // namespace tbg
