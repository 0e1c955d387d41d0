// In-situ SL step through a time-dependent velocity: a set of up to four
// velocity trees blended with per-stage weights -- the reference's
// FieldSetFunctor (cubic interpolation in time of four trees,
// src/tree/tree_set_functor.h:49-72, src/utils/cubic.h:42-56) and
// FieldExtrapFunctor (1.5 v_n - 0.5 v_{n-1}, src/tree/tree_extrap_functor.h:
// 47-78) as IntegrateRK2 calls them at each stage (src/semilag/traj.inc:
// 20-45, :71-93).  This is the general kernel, instantiated per degree by
// tv_deg_*.cu: every tree is evaluated at every stage point in FP64 and the
// values blended, so the trees may have different leaf structures; the
// first stage, at the target node, comes from each tree's node-grid pass.
// In the double-float mode, trees of one structure take the fast path in
// capi.cu instead (blended coefficients through the fused step).
#pragma once

#include "tree_kernels.cuh"

namespace tbg {

// SAME (the trees share their leaves): one leaf lookup and one set of T_k per
// point serve every tree -- what each tree's eval_point would compute, so the
// values are the same bits.
template <int D, bool SAME>
__device__ __forceinline__ void tv_velocity(const TvArgs& a, int stage, double& x, double& y,
                                            double& z, bool per, double (&v)[3]) {
  constexpr int NC = D * (D + 1) * (D + 2) / 6;
  const double* w = a.w + stage * a.m;
  v[0] = v[1] = v[2] = 0.0;
  if constexpr (SAME) {
    if (per) wrap3(x, y, z);
    const bool in = inside(x, y, z, per);
    double tx[D], ty[D], tz[D];
    int64_t leaf = 0;
    if (in) {
      leaf = find_leaf(a.vel[0], morton3(quantise(x), quantise(y), quantise(z)));
      const Geom g = load_geom(a.vel[0].geom + leaf);
      cheb_T<D>((x - g.x) * g.w - 1.0, tx);
      cheb_T<D>((y - g.y) * g.w - 1.0, ty);
      cheb_T<D>((z - g.z) * g.w - 1.0, tz);
    }
    for (int k = 0; k < a.m; ++k) {
      double u[3] = {0.0, 0.0, 0.0};
      if (in) {
        const double* c = a.vel[k].coeff + leaf * a.vel[k].stride;
#pragma unroll
        for (int l = 0; l < 3; ++l) u[l] = tri_sum<D>(GlobalLoad{c + l * NC}, tx, ty, tz);
      }
      v[0] = fma(w[k], u[0], v[0]);
      v[1] = fma(w[k], u[1], v[1]);
      v[2] = fma(w[k], u[2], v[2]);
    }
  } else {
    for (int k = 0; k < a.m; ++k) {
      double u[3];
      eval_point<D, 3>(a.vel[k], x, y, z, per, u);  // wraps the point in place
      v[0] = fma(w[k], u[0], v[0]);
      v[1] = fma(w[k], u[1], v[1]);
      v[2] = fma(w[k], u[2], v[2]);
    }
  }
}

template <int D, bool SAME>
__global__ void __launch_bounds__(128) k_semilag_tv(const TvArgs a) {
  constexpr int NP = D * D * D;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= a.con.L * NP) return;
  const int64_t leaf = t / NP;
  const int p = (int)(t - leaf * NP);
  const Geom g = load_geom(a.con.geom + leaf);
  const double h = leaf_side(g);
  double x = g.x + h * a.nodes.x[p % D];
  double y = g.y + h * a.nodes.x[(p / D) % D];
  double z = g.z + h * a.nodes.x[p / (D * D)];
  const bool per = a.periodic != 0;
  const double half_tau = 0.5 * a.tau;
#pragma unroll 1
  for (int s = 0; s < a.nrk; ++s) {
    double v[3];
    if (s == 0 && a.vn) {
      // the trees' values at the target node from the node-grid pass, blended
      // in the order tv_velocity blends them; X wrapped as eval_point wraps it
      if (per) {
        x = wrap1(x);
        y = wrap1(y);
        z = wrap1(z);
      }
      const int64_t N = a.con.L * NP;
      // a shared upper-face node takes its neighbour's node values (the
      // same point; the node-grid pass left it unwritten)
      const int32_t f = a.face ? __ldg(a.face + t) : -1;
      const int64_t tv = f >= 0 ? (int64_t)f : t;
      v[0] = v[1] = v[2] = 0.0;
      for (int k = 0; k < a.m; ++k) {
        const double* u = a.vn + 3 * (k * N + tv);
        v[0] = fma(a.w[k], __ldg(u + 0), v[0]);
        v[1] = fma(a.w[k], __ldg(u + 1), v[1]);
        v[2] = fma(a.w[k], __ldg(u + 2), v[2]);
      }
    } else {
      tv_velocity<D, SAME>(a, 2 * s, x, y, z, per, v);  // at X (wrapped in place)
    }
    double px = fma(half_tau, v[0], x), py = fma(half_tau, v[1], y),
           pz = fma(half_tau, v[2], z);
    tv_velocity<D, SAME>(a, 2 * s + 1, px, py, pz, per, v);  // at X*
    x = fma(a.tau, v[0], x);
    y = fma(a.tau, v[1], y);
    z = fma(a.tau, v[2], z);
  }
  double c[1];
  eval_point<D, 1>(a.con, x, y, z, per, c);
  a.vals[t] = c[0];
}

template <int D>
void launch_semilag_tv(const TvArgs& a, cudaStream_t s) {
  const int64_t n = a.con.L * D * D * D;
  if (n <= 0) return;
  const unsigned blocks = (unsigned)((n + 127) / 128);
  if (a.same_leaves)
    k_semilag_tv<D, true><<<blocks, 128, 0, s>>>(a);
  else
    k_semilag_tv<D, false><<<blocks, 128, 0, s>>>(a);
}

}  // namespace tbg
