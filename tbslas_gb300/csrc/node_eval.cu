// A tree evaluated at every Chebyshev node of another tree's leaves -- the
// velocity at the targets X that the first RK2 stage of the in-situ SL step
// needs (SolveSemilagInSitu collects the nodes, src/tree/tree_semilag.h:
// 114-124, and IntegrateRK2 evaluates the velocity functor there first,
// src/semilag/traj.inc:20-68).
//
// Pointwise, each of the D^3 nodes of a destination leaf costs a Chebyshev
// sum of Nc = D(D+1)(D+2)/6 terms per component.  The nodes form a tensor
// grid, and the part of it inside one source leaf is a tensor sub-grid, so
// the sums factor (sum factorisation):
//   w(i,j,a) = sum_k c[i][j][k] T_k(x_a)          Nc * na
//   v(i,b,a) = sum_j T_j(y_b) w(i,j,a)            D(D+1)/2 * nb * na
//   u(c,b,a) = sum_i T_i(z_c) v(i,b,a)            D * nc * nb * na
// ~(1/6 + 1/2 + 1) D^4 per leaf and component instead of D^3 Nc.  These are
// tri_sum's nested sums with the same fma order, the same T_k recurrences
// and the same node and local coordinates, so every value is bit-identical to
// the pointwise FP64 evaluation (eval_point).
//
// One CTA per destination leaf: each node's source leaf is found by the
// usual key search (points outside the domain evaluate to 0); then, source
// leaf by source leaf, the sub-grid of nodes it holds is evaluated with the
// three passes in shared memory.  Runtime degree; FP64 (FP64 pipe).
#include <atomic>
#include <climits>
#include <cstring>
#include <vector>

#include "host_cheb.h"

#include "internal.h"

namespace tbg {

namespace {

constexpr int kNodeEvalThreads = 256;

__device__ __forceinline__ void cheb_T_rt(double xi, int D, double* T, int stride) {
  // the operations of cheb_T<D>, with a runtime length
  const bool ok = fabs(xi) <= 1.0;
  const double x = ok ? xi : 0.0;
  const double t0 = ok ? 1.0 : 0.0;
  T[0] = t0;
  if (D > 1) T[stride] = x;
  const double x2 = 2.0 * x;
  double a = t0, b = x;
  for (int k = 2; k < D; ++k) {
    const double t = fma(x2, b, -a);
    T[k * stride] = t;
    a = b;
    b = t;
  }
}

__host__ __device__ constexpr size_t node_eval_smem(int Ds, int Dd) {
  // doubles: coordinates 3*Dd, T tables 3*Ds*Dd, w: Ds(Ds+1)/2*Dd, v: Ds*Dd*Dd;
  // ints: leaf per node Dd^3, index lists 3*Dd
  return (size_t)(3 * Dd + 3 * Ds * Dd + Ds * (Ds + 1) / 2 * Dd + Ds * Dd * Dd) * 8 +
         (size_t)(Dd * Dd * Dd + 3 * Dd) * 4;
}

// One destination leaf (the whole CTA).  out: the destination tree's
// [L * Dd^3][src.dof] array.
__device__ __forceinline__ void eval_on_nodes_leaf(const TreeView& S, const TreeView& dst,
                                                   const Nodes1D& nodes, bool per, int64_t leaf,
                                                   double* __restrict__ out_all, double* sm) {
  __shared__ int s_first;
  __shared__ unsigned s_mask[3];
  __shared__ int s_n[3];
  const int Ds = S.q + 1, Dd = dst.q + 1, Dd2 = Dd * Dd, Dd3 = Dd2 * Dd;
  const int NCs = Ds * (Ds + 1) * (Ds + 2) / 6, dof = S.dof;
  const int tid = threadIdx.x, bs = blockDim.x;

  double* sx = sm;                       // [3][Dd] wrapped node coordinates
  double* sT = sx + 3 * Dd;              // [3][Ds][Dd]: T_k of the listed indices
  double* sw = sT + 3 * Ds * Dd;         // [pair(i,j)][Dd]
  double* sv = sw + Ds * (Ds + 1) / 2 * Dd;  // [i][Dd][Dd]
  int* sleaf = reinterpret_cast<int*>(sv + Ds * Dd * Dd);  // [Dd^3]
  int* sidx = sleaf + Dd3;               // [3][Dd] index lists

  const Geom g = load_geom(dst.geom + leaf);
  const double h = 2.0 / g.w;
  if (tid < 3 * Dd) {
    const int ax = tid / Dd, i = tid - ax * Dd;
    const double o = ax == 0 ? g.x : (ax == 1 ? g.y : g.z);
    double c = o + h * nodes.x[i];
    if (per) c = wrap1(c);
    sx[tid] = c;
  }
  __syncthreads();
  double* out = out_all + leaf * (int64_t)Dd3 * dof;
  for (int p = tid; p < Dd3; p += bs) {
    const double x = sx[p % Dd], y = sx[Dd + (p / Dd) % Dd], z = sx[2 * Dd + p / Dd2];
    if (inside(x, y, z, per)) {
      sleaf[p] = (int)find_leaf(S, morton3(quantise(x), quantise(y), quantise(z)));
    } else {
      sleaf[p] = -1;
      for (int l = 0; l < dof; ++l) out[(int64_t)p * dof + l] = 0.0;
    }
  }
  __syncthreads();

  for (;;) {
    if (tid == 0) s_first = INT_MAX;
    if (tid < 3) s_mask[tid] = 0u;
    __syncthreads();
    int first = INT_MAX;
    for (int p = tid; p < Dd3; p += bs)
      if (sleaf[p] >= 0) {
        first = p;
        break;
      }
    if (first != INT_MAX) atomicMin(&s_first, first);
    __syncthreads();
    if (s_first == INT_MAX) break;
    const int V = sleaf[s_first];
    for (int p = tid; p < Dd3; p += bs)
      if (sleaf[p] == V) {
        atomicOr(&s_mask[0], 1u << (p % Dd));
        atomicOr(&s_mask[1], 1u << ((p / Dd) % Dd));
        atomicOr(&s_mask[2], 1u << (p / Dd2));
      }
    __syncthreads();
    if (tid < 3) {
      int n = 0;
      for (int i = 0; i < Dd; ++i)
        if (s_mask[tid] >> i & 1u) sidx[tid * Dd + n++] = i;
      s_n[tid] = n;
    }
    __syncthreads();
    const int na = s_n[0], nb = s_n[1], nz = s_n[2];
    const Geom vg = load_geom(S.geom + V);
    // T tables of the listed indices: sT[ax][k][i'] (the local coordinate
    // and recurrence of eval_point)
    if (tid < 3 * Dd) {
      const int ax = tid / Dd, i = tid - ax * Dd;
      const int n = ax == 0 ? na : (ax == 1 ? nb : nz);
      if (i < n) {
        const double c = sx[ax * Dd + sidx[ax * Dd + i]];
        const double o = ax == 0 ? vg.x : (ax == 1 ? vg.y : vg.z);
        cheb_T_rt((c - o) * vg.w - 1.0, Ds, sT + ax * Ds * Dd + i, Dd);
      }
    }
    __syncthreads();
    const double* Tx = sT;
    const double* Ty = sT + Ds * Dd;
    const double* Tz = sT + 2 * Ds * Dd;
    const int npair = Ds * (Ds + 1) / 2;
    for (int l = 0; l < dof; ++l) {
      const double* c = S.coeff + (int64_t)V * S.stride + (int64_t)l * NCs;
      // w(i,j,a') = sum_k c[i][j][k] T_k(x_a')
      for (int o = tid; o < npair * na; o += bs) {
        const int pr = o / na, ai = o - pr * na;
        // pair index pr -> (i, j): rows of length Ds - i
        int i = 0, rem = pr;
        while (rem >= Ds - i) {
          rem -= Ds - i;
          ++i;
        }
        const int j = rem;
        const int m = Ds - i;
        const int base = NCs - m * (m + 1) * (m + 2) / 6 + j * m - (j * (j - 1)) / 2;
        double w = 0.0;
        for (int k = 0; k < m - j; ++k) w = fma(__ldg(c + base + k), Tx[k * Dd + ai], w);
        sw[pr * Dd + ai] = w;
      }
      __syncthreads();
      // v(i,b',a') = sum_j T_j(y_b') w(i,j,a')
      for (int o = tid; o < Ds * nb * na; o += bs) {
        const int ai = o % na, bi = (o / na) % nb, i = o / (na * nb);
        const int prow = i * Ds - (i * (i - 1)) / 2;  // pair index of (i, 0)
        double v = 0.0;
        for (int j = 0; j < Ds - i; ++j) v = fma(Ty[j * Dd + bi], sw[(prow + j) * Dd + ai], v);
        sv[(i * Dd + bi) * Dd + ai] = v;
      }
      __syncthreads();
      // u(c',b',a') = sum_i T_i(z_c') v(i,b',a'), kept where the node's leaf is V
      for (int o = tid; o < nz * nb * na; o += bs) {
        const int ai = o % na, bi = (o / na) % nb, ci = o / (na * nb);
        const int p = sidx[ai] + Dd * (sidx[Dd + bi] + Dd * sidx[2 * Dd + ci]);
        if (sleaf[p] != V) continue;
        double u = 0.0;
        for (int i = 0; i < Ds; ++i) u = fma(Tz[i * Dd + ci], sv[(i * Dd + bi) * Dd + ai], u);
        out[(int64_t)p * dof + l] = u;
      }
      __syncthreads();
    }
    for (int p = tid; p < Dd3; p += bs)
      if (sleaf[p] == V) sleaf[p] = -2;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kNodeEvalThreads) k_eval_on_nodes(const NodeEvalJob j,
                                                                    int periodic) {
  extern __shared__ __align__(16) double sm[];
  eval_on_nodes_leaf(j.src, j.dst, j.nodes, periodic != 0, blockIdx.x, j.out, sm);
}

// Batched: one CTA per (job, destination leaf) item.
__global__ void __launch_bounds__(kNodeEvalThreads) k_batch_eval_on_nodes(
    const NodeEvalJob* __restrict__ jobs, const NodeEvalItem* __restrict__ items, int periodic) {
  extern __shared__ __align__(16) double sm[];
  __shared__ NodeEvalJob sj;
  const NodeEvalItem it = items[blockIdx.x];
  if (threadIdx.x == 0) sj = jobs[it.job];
  __syncthreads();
  eval_on_nodes_leaf(sj.src, sj.dst, sj.nodes, periodic != 0, it.leaf, sj.out, sm);
}

void allow_node_smem(const void* kernel, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (!(done.load() & bit)) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)node_eval_smem(TBSLAS_MAX_DEGREE + 1, TBSLAS_MAX_DEGREE + 1));
    done.fetch_or(bit);
  }
}

std::atomic<uint64_t> g_smem_nodes{0}, g_smem_batch_nodes{0};

}  // namespace

void launch_eval_on_nodes(const TreeView& src, const TreeView& dst, int periodic, double* out,
                          cudaStream_t s) {
  if (dst.L <= 0) return;
  NodeEvalJob j;
  j.src = src;
  j.dst = dst;
  std::memset(&j.nodes, 0, sizeof(j.nodes));
  const std::vector<double> x = cheb_nodes_1d(dst.q);
  for (int i = 0; i <= dst.q; ++i) j.nodes.x[i] = x[i];
  j.out = out;
  allow_node_smem((const void*)k_eval_on_nodes, g_smem_nodes);
  k_eval_on_nodes<<<(unsigned)dst.L, kNodeEvalThreads, node_eval_smem(src.q + 1, dst.q + 1),
                    s>>>(j, periodic);
}

void launch_batch_eval_on_nodes(const NodeEvalJob* jobs, const NodeEvalItem* items,
                                int64_t n_items, int max_q, int periodic, cudaStream_t s) {
  if (n_items <= 0) return;
  allow_node_smem((const void*)k_batch_eval_on_nodes, g_smem_batch_nodes);
  k_batch_eval_on_nodes<<<(unsigned)n_items, kNodeEvalThreads,
                          node_eval_smem(max_q + 1, max_q + 1), s>>>(jobs, items, periodic);
}

}  // namespace tbg
