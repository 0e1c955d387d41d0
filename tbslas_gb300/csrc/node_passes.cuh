// Sum-factorised evaluation of a tree leaf's expansion on a tensor sub-grid
// of a destination leaf's Chebyshev nodes, shared by the node-grid
// evaluation (node_eval.cu) and the re-meshing transfer (remesh.cu).
#pragma once

#include "internal.h"

namespace tbg {

template <int Ds>
__device__ __forceinline__ void cheb_T_col(double xi, double* T, int stride) {
  // the operations of cheb_T<Ds>, written to a strided column
  const bool ok = abs_at_most_one(xi);
  const double x = ok ? xi : 0.0;
  const double t0 = ok ? 1.0 : 0.0;
  T[0] = t0;
  if (Ds > 1) T[stride] = x;
  const double x2 = twice(x);
  double a = t0, b = x;
#pragma unroll
  for (int k = 2; k < Ds; ++k) {
    const double t = fma(x2, b, -a);
    T[k * stride] = t;
    a = b;
    b = t;
  }
}

// The part of a destination leaf's node grid inside one source leaf: leaf
// V, the listed node indices per axis (sidx[ax*Dd + i'], i' < n[ax]) and
// T_k of their local coordinates in V (T[ax][k][i'], stride Dd).
struct SubGrid {
  int64_t V;
  int na, nb, nz;
  const int* sidx;
  const double *Tx, *Ty, *Tz;
};

// The source expansion at every node of the sub-grid, by the three passes
//   w(l; i,j,a') = sum_k c[l][i][j][k] T_k(x_a')
//   v(i)         = sum_j T_j(y_b') w(l; i,j,a')        (per column l, b', a')
//   u(c')        = sum_i T_i(z_c') v(i)
// -- tri_sum's nested sums with its fma order (the T_0 terms by fma_t0), so
// each value is bit-identical to eval_point.  ncomp components: coeff(l) is
// component l's Nc coefficients in the sub-grid's source leaf, out(l) its
// output, node p = a + Dd (b + Dd c) at out(l)[p * pstride].  sw: ncomp *
// Ds (Ds + 1) / 2 * Dd doubles of shared memory.  All threads of the block
// call it; it contains a barrier between the first two passes.
template <int Ds, class CoeffOf, class OutOf>
__device__ __forceinline__ void eval_subgrid_comps(const SubGrid& sg, int Dd, int ncomp,
                                                   CoeffOf coeff, OutOf outp, int64_t pstride,
                                                   double* sw) {
  constexpr int NCs = Ds * (Ds + 1) * (Ds + 2) / 6, npair = Ds * (Ds + 1) / 2;
  const int Dd2 = Dd * Dd;
  const int tid = threadIdx.x, bs = blockDim.x;
  const int na = sg.na, nb = sg.nb, nz = sg.nz;
  const int* sidx = sg.sidx;
  // items (a', l, pair) with the pair slowest: the lanes of a warp share
  // one row length (the k loop) instead of diverging over several
  for (int o = tid; o < ncomp * npair * na; o += bs) {
    const int ai = o % na, r = o / na, l = r % ncomp, pr = r / ncomp;
    int i = 0, rem = pr;  // pair index -> (i, j): rows of length Ds - i
    while (rem >= Ds - i) {
      rem -= Ds - i;
      ++i;
    }
    const int j = rem, m = Ds - i;
    const double* c = coeff(l) + (NCs - m * (m + 1) * (m + 2) / 6 + j * m - (j * (j - 1)) / 2);
    double w = fma_t0(sg.Tx[ai], __ldg(c));  // T_0 term, as tri_sum
    for (int k = 1; k < m - j; ++k) w = fma(__ldg(c + k), sg.Tx[k * Dd + ai], w);
    sw[(l * npair + pr) * Dd + ai] = w;
  }
  __syncthreads();
  for (int o = tid; o < ncomp * nb * na; o += bs) {
    const int ai = o % na, r = o / na, bi = r % nb, l = r / nb;
    const double* wl = sw + l * npair * Dd + ai;
    double v[Ds];
    int prow = 0;
#pragma unroll
    for (int i = 0; i < Ds; ++i) {
      double s = fma_t0(sg.Ty[bi], wl[prow * Dd]);
#pragma unroll
      for (int j = 1; j < Ds - i; ++j) s = fma(sg.Ty[j * Dd + bi], wl[(prow + j) * Dd], s);
      v[i] = s;
      prow += Ds - i;
    }
    const int pab = sidx[ai] + Dd * sidx[Dd + bi];
    double* ol = outp(l);
    for (int ci = 0; ci < nz; ++ci) {
      double u = fma_t0(sg.Tz[ci], v[0]);
#pragma unroll
      for (int i = 1; i < Ds; ++i) u = fma(sg.Tz[i * Dd + ci], v[i], u);
      ol[(int64_t)(pab + Dd2 * sidx[2 * Dd + ci]) * pstride] = u;
    }
  }
}

// The S.dof components of tree S's leaf sg.V; component l of node p goes to
// out[p * pstride + l * lstride].
template <int Ds>
__device__ __forceinline__ void eval_subgrid(const TreeView& S, const SubGrid& sg, int Dd,
                                             double* __restrict__ out, int64_t pstride,
                                             int64_t lstride, double* sw) {
  constexpr int NCs = Ds * (Ds + 1) * (Ds + 2) / 6;
  const double* cV = S.coeff + sg.V * S.stride;
  eval_subgrid_comps<Ds>(
      sg, Dd, S.dof, [=](int l) { return cV + l * NCs; },
      [=](int l) { return out + l * lstride; }, pstride, sw);
}

}  // namespace tbg
