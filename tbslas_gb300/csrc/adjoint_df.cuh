// The adjoint step of adjoint_kernels.cuh with its sums in double-float
// (df64.cuh): the two gradient sums (grad c^k at Xd, grad(g . v) at X*) and
// the three CTA-cooperative scatters run as hi/lo float pairs on the FP32
// pipe; point locations, T_k and dT_k recurrences, the weights and the global
// accumulation (FP64 atomics) stay FP64.  The checkpointed points are the
// FP64 forward's, so every leaf choice is the FP64 adjoint's and results
// differ from it by the sums' rounding (~1e-15 relative).
#pragma once

#include "adjoint_kernels.cuh"

namespace tbg {

// Targets (threads) per CTA of the double-float adjoint: 192 gives every warp
// one coefficient per scatter pass at q = 8 (Nc = 165); with 128 threads two
// warps carried a second coefficient and set the pace (measured on GB300,
// q = 8: 36.0 -> 34.0 ms per 4-step adjoint pass of a 4096-leaf tree).
constexpr int kAdjDfThreads = 192;

// Per-thread shared-memory slots of the gradient sums, 4*D elements: T_j(y),
// dT_j(y), T_i(z), dT_i(z) (ThreadSlots: element k at s[k * blockDim]).
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

// Staging of one block's points for a double-float scatter: per point the
// x, y, z Chebyshev values, up to three weights and the leaf.
template <int D>
struct AdjStageDF {
  float2 tx[kAdjDfThreads][D];
  float2 ty[kAdjDfThreads][D];
  float2 tz[kAdjDfThreads][D];
  float2 w[kAdjDfThreads][3];
  long long leaf[kAdjDfThreads];
  long long cur;
};

template <int D>
constexpr size_t adj_df_smem() {
  const size_t stage = sizeof(AdjStageDF<D>);
  const size_t slots = (size_t)4 * D * kAdjDfThreads * sizeof(float2);
  return stage > slots ? stage : slots;
}

// out[leaf*stride + l*NC + n] += w[l] * phi_n(point) for every thread's point
// (leaf < 0: none); the thread's coefficients n = tid + c*blockDim are
// carried together through one pass over the block's points of each leaf.
template <int D, int DOF>
__device__ __forceinline__ void cta_scatter_df(AdjStageDF<D>& sm, double* __restrict__ out,
                                               int64_t stride, int64_t leaf,
                                               const double (&w)[DOF], const double (&tx)[D],
                                               const double (&ty)[D], const double (&tz)[D]) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  constexpr int PER = (NC + kAdjDfThreads - 1) / kAdjDfThreads;
  const int tid = threadIdx.x;
  __syncthreads();  // the staging area is free
  sm.leaf[tid] = leaf;
  if (leaf >= 0) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const df a = df_split_bits(tx[k]), b = df_split_bits(ty[k]), c = df_split_bits(tz[k]);
      sm.tx[tid][k] = make_float2(a.hi, a.lo);
      sm.ty[tid][k] = make_float2(b.hi, b.lo);
      sm.tz[tid][k] = make_float2(c.hi, c.lo);
    }
#pragma unroll
    for (int l = 0; l < DOF; ++l) {
      const df v = df_from_double(w[l]);
      sm.w[tid][l] = make_float2(v.hi, v.lo);
    }
  }
  int mi[PER], mj[PER], mk[PER];
#pragma unroll
  for (int c = 0; c < PER; ++c) {
    const int n = tid + c * kAdjDfThreads;
    int idx = 0;
    mi[c] = -1;
    mj[c] = mk[c] = 0;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D - i; ++j) {
        const int len = D - i - j;
        if (n >= idx && n < idx + len) {
          mi[c] = i;
          mj[c] = j;
          mk[c] = n - idx;
        }
        idx += len;
      }
  }
  __syncthreads();
  for (;;) {
    if (tid < 32) {
      long long first = -1;
#pragma unroll
      for (int chunk = 0; chunk < kAdjDfThreads / 32; ++chunk) {
        const long long v = sm.leaf[chunk * 32 + tid];
        const unsigned m = __ballot_sync(0xffffffffu, v >= 0);
        if (m) {
          first = __shfl_sync(0xffffffffu, v, __ffs(m) - 1);
          break;
        }
      }
      if (tid == 0) sm.cur = first;
    }
    __syncthreads();
    const long long cur = sm.cur;
    if (cur < 0) break;
    df acc[PER][DOF];
#pragma unroll
    for (int c = 0; c < PER; ++c)
#pragma unroll
      for (int l = 0; l < DOF; ++l) acc[c][l] = df{0.f, 0.f};
    for (int p = 0; p < kAdjDfThreads; ++p) {
      if (sm.leaf[p] != cur) continue;
      df wp[DOF];
#pragma unroll
      for (int l = 0; l < DOF; ++l) wp[l] = df{sm.w[p][l].x, sm.w[p][l].y};
#pragma unroll
      for (int c = 0; c < PER; ++c) {
        if (mi[c] < 0) continue;
        const float2 a = sm.tz[p][mi[c]], b = sm.ty[p][mj[c]], e = sm.tx[p][mk[c]];
        const df t = df_mul(df_mul(df{a.x, a.y}, df{b.x, b.y}), df{e.x, e.y});
#pragma unroll
        for (int l = 0; l < DOF; ++l) df_fma_acc(acc[c][l], wp[l], t);
      }
    }
#pragma unroll
    for (int c = 0; c < PER; ++c) {
      if (mi[c] < 0) continue;
      const int n = tid + c * kAdjDfThreads;
#pragma unroll
      for (int l = 0; l < DOF; ++l) {
        const double v = df_to_double(df_norm(acc[c][l]));
        if (v != 0.0) atomicAdd(out + cur * stride + l * NC + n, v);
      }
    }
    __syncthreads();
    if (sm.leaf[tid] == cur) sm.leaf[tid] = -1;
    __syncthreads();
  }
}

// Four (q <= 8) or three CTAs per SM: with the register cap the kernel
// spills a little but keeps 24 or 18 warps resident.
template <int D>
__global__ void __launch_bounds__(kAdjDfThreads, (D <= 9 ? 4 : 3)) k_adjoint_df(const AdjArgs a,
                                                            const float2* __restrict__ con2) {
  constexpr int NP = D * D * D;
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  extern __shared__ __align__(16) unsigned char adj_df_raw[];
  AdjStageDF<D>& sm = *reinterpret_cast<AdjStageDF<D>*>(adj_df_raw);
  const ThreadSlots slots{reinterpret_cast<float2*>(adj_df_raw) + threadIdx.x, kAdjDfThreads};
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < a.con.L * NP;
  const bool per = a.periodic != 0;
  const int64_t tt = active ? t : 0;
  const int64_t leaf = tt / NP;
  const int p = (int)(tt - leaf * NP);
  const Geom gl = load_geom(a.con.geom + leaf);
  const double h = 2.0 / gl.w;
  double x = gl.x + h * a.nodes.x[p % D];
  double y = gl.y + h * a.nodes.x[(p / D) % D];
  double z = gl.z + h * a.nodes.x[p / (D * D)];
  double xs, ys, zs, xd, yd, zd;
  if (a.xmid) {
    xs = a.xmid[3 * tt];
    ys = a.xmid[3 * tt + 1];
    zs = a.xmid[3 * tt + 2];
    xd = a.xdep[3 * tt];
    yd = a.xdep[3 * tt + 1];
    zd = a.xdep[3 * tt + 2];
  } else if (a.vn) {
    // recompute from the node-grid velocity (bit-identical to eval_point at X)
    double v[3];
    double px = x, py = y, pz = z;
    if (per) {
      px = wrap1(px);
      py = wrap1(py);
      pz = wrap1(pz);
    }
    xs = fma(0.5 * a.tau, __ldg(a.vn + 3 * tt + 0), px);
    ys = fma(0.5 * a.tau, __ldg(a.vn + 3 * tt + 1), py);
    zs = fma(0.5 * a.tau, __ldg(a.vn + 3 * tt + 2), pz);
    double qx = xs, qy = ys, qz = zs;
    eval_point<D, 3>(a.vel, qx, qy, qz, per, v);
    xd = fma(a.tau, v[0], px);
    yd = fma(a.tau, v[1], py);
    zd = fma(a.tau, v[2], pz);
  } else {
    double v[3];
    double px = x, py = y, pz = z;
    eval_point<D, 3>(a.vel, px, py, pz, per, v);
    xs = fma(0.5 * a.tau, v[0], px);
    ys = fma(0.5 * a.tau, v[1], py);
    zs = fma(0.5 * a.tau, v[2], pz);
    double qx = xs, qy = ys, qz = zs;
    eval_point<D, 3>(a.vel, qx, qy, qz, per, v);
    xd = fma(a.tau, v[0], px);
    yd = fma(a.tau, v[1], py);
    zd = fma(a.tau, v[2], pz);
  }
  const double mu = active ? a.mu[tt] : 0.0;

  // g = mu grad c^k(Xd); lambda^k += mu phi(Xd)
  double gvec[3] = {0.0, 0.0, 0.0};
  {
    Geom g;
    int64_t lf = locate<D>(a.con, xd, yd, zd, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D];
    if (lf >= 0) {
      df dtx[D], ddx[D];
      grad_tables<D>(g, xd, yd, zd, dtx, ddx, slots);
      double gr[3];
      tri_grad_df<D>(GradOne{con2 + lf * NC}, dtx, ddx, slots, gr);
      gvec[0] = mu * gr[0] * g.w;
      gvec[1] = mu * gr[1] * g.w;
      gvec[2] = mu * gr[2] * g.w;
      cheb_T<D>((xd - g.x) * g.w - 1.0, tx);
      cheb_T<D>((yd - g.y) * g.w - 1.0, ty);
      cheb_T<D>((zd - g.z) * g.w - 1.0, tz);
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) tx[k] = ty[k] = tz[k] = 0.0;
    }
    const double w[1] = {mu};
    cta_scatter_df<D, 1>(sm, a.lambda, NC, lf, w, tx, ty, tz);
  }
  // tau g (x) phi(X*) and J_v(X*)^T g = grad(g . v)(X*)
  double jtg[3] = {0.0, 0.0, 0.0};
  {
    Geom g;
    int64_t lf = locate<D>(a.vel, xs, ys, zs, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D];
    if (lf >= 0) {
      df dtx[D], ddx[D];
      grad_tables<D>(g, xs, ys, zs, dtx, ddx, slots);
      double gr[3];
      tri_grad_df<D>(GradW3{a.vel.coeff2 + lf * a.vel.stride, NC, df_from_double(gvec[0]),
                            df_from_double(gvec[1]), df_from_double(gvec[2])},
                     dtx, ddx, slots, gr);
      jtg[0] = gr[0] * g.w;
      jtg[1] = gr[1] * g.w;
      jtg[2] = gr[2] * g.w;
      cheb_T<D>((xs - g.x) * g.w - 1.0, tx);
      cheb_T<D>((ys - g.y) * g.w - 1.0, ty);
      cheb_T<D>((zs - g.z) * g.w - 1.0, tz);
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) tx[k] = ty[k] = tz[k] = 0.0;
    }
    const double w[3] = {a.tau * gvec[0], a.tau * gvec[1], a.tau * gvec[2]};
    cta_scatter_df<D, 3>(sm, a.grad_vel, 3 * NC, lf, w, tx, ty, tz);
  }
  // tau^2/2 J_v(X*)^T g (x) phi(X): X is a node, so the weights go to the
  // node-grid scatter when a buffer is given
  if (a.wnode) {
    const double c2 = 0.5 * a.tau * a.tau;
    if (active) {
      a.wnode[3 * t + 0] = c2 * jtg[0];
      a.wnode[3 * t + 1] = c2 * jtg[1];
      a.wnode[3 * t + 2] = c2 * jtg[2];
    }
    return;
  }
  {
    Geom g;
    int64_t lf = locate<D>(a.vel, x, y, z, per, g);
    if (!active) lf = -1;
    double tx[D], ty[D], tz[D];
    if (lf >= 0) {
      cheb_T<D>((x - g.x) * g.w - 1.0, tx);
      cheb_T<D>((y - g.y) * g.w - 1.0, ty);
      cheb_T<D>((z - g.z) * g.w - 1.0, tz);
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) tx[k] = ty[k] = tz[k] = 0.0;
    }
    const double c2 = 0.5 * a.tau * a.tau;
    const double w[3] = {c2 * jtg[0], c2 * jtg[1], c2 * jtg[2]};
    cta_scatter_df<D, 3>(sm, a.grad_vel, 3 * NC, lf, w, tx, ty, tz);
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
void register_adjoint_degree(CkptFn* c, AdjFn* a, AdjDfFn* d) {
  c[D - 1] = &launch_ckpt<D>;
  a[D - 1] = &launch_adjoint<D>;
  d[D - 1] = &launch_adjoint_df<D>;
}

}  // namespace tbg
