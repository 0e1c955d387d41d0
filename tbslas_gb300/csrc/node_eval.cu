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
// Neighbouring leaves of one depth share their face nodes (the stretched end
// nodes are exactly 0 and 1 at most degrees): a leaf's shared upper-face
// nodes are not evaluated but copied from the neighbour afterwards.  Which
// nodes those are depends only on the destination tree's leaves, so the map
// (face_source per node) is built once per leaf structure and boundary
// condition (k_face_map) and read by every evaluation.
//
// One CTA per destination leaf.  Leaves tile the unit cube (tree_create
// checks it), so the nodes a source leaf holds are those inside its box:
// starting from the first node not yet evaluated, one key search finds its
// source leaf, per-axis box tests give the sub-grid, and the three passes
// evaluate it -- w in shared memory, then per (b, a) column v(., b, a) in
// registers and every u of the column.  FP64 (FP64 pipe); templated on the
// source degree (register arrays), runtime destination degree.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstring>
#include <vector>

#include "host_cheb.h"
#include "internal.h"
#include "node_passes.cuh"

namespace tbg {

namespace {

constexpr int kNodeEvalThreads = 256;

// Arithmetic of the transposed passes: FP64, or double-float pairs
// accumulated with df_fma_acc (df64.cuh).
struct NodeF64 {
  typedef double T;
  __device__ static T zero() { return 0.0; }
  __device__ static void mac(T& acc, T a, T b) { acc = fma(a, b, acc); }
  __device__ static T done(T acc) { return acc; }
  __device__ static T from(double x) { return x; }
  __device__ static double value(T v) { return v; }
};
struct NodeDF {
  typedef float2 T;
  __device__ static T zero() { return make_float2(0.f, 0.f); }
  __device__ static void mac(T& acc, T a, T b) {
    df s{acc.x, acc.y};
    df_fma_acc(s, df{a.x, a.y}, df{b.x, b.y});
    acc = make_float2(s.hi, s.lo);
  }
  __device__ static T done(T acc) {
    const df v = df_norm(df{acc.x, acc.y});
    return make_float2(v.hi, v.lo);
  }
  __device__ static T from(double x) {
    const df v = df_from_double(x);
    return make_float2(v.hi, v.lo);
  }
  __device__ static double value(T v) { return df_to_double(df_norm(df{v.x, v.y})); }
};

// Shared memory of the sub-grid walk: coordinates 3*Dd and T tables
// 3*Ds*Dd (doubles), quantised coordinates and index lists 6*Dd (ints), the
// node state Dd^3 (bytes); then the pass buffers of the caller.
__host__ __device__ constexpr size_t walk_smem(int Ds, int Dd) {
  return (size_t)(3 * Dd + 3 * Ds * Dd) * 8 + (size_t)(6 * Dd) * 4 +
         (size_t)(Dd * Dd * Dd + 15) / 16 * 16;
}
__host__ __device__ constexpr size_t node_eval_smem(int Ds, int Dd, int dof) {
  return walk_smem(Ds, Dd) + (size_t)dof * Ds * (Ds + 1) / 2 * Dd * 8;  // w
}
__host__ __device__ constexpr size_t node_scatter_smem(int Ds, int Dd, int dof) {
  (void)dof;
  return walk_smem(Ds, Dd) +
         (size_t)(3 * Ds * Dd + Dd * Dd * Dd + Ds * Dd * Dd + Ds * (Ds + 1) / 2 * Dd) *
             8;  // T (pass arithmetic), W, H, G
}

// Node (a, b, c) of destination leaf `leaf` on an upper face, where its
// point is also a node of the neighbouring destination leaf of the same
// depth that contains it (the stretched end nodes are exactly 0 and 1, so
// neighbours share face nodes): returns that node's target index -- the
// neighbour's node with the upper-face indices set to 0, which is not itself
// on an upper face -- or -1.  The point is the same double, so its source
// leaf and value are the same.
__device__ __forceinline__ int64_t face_source(const TreeView& dst, const Nodes1D& nodes, bool per,
                                               int64_t leaf, const Geom& g, int a, int b, int c) {
  const int Dd = dst.q + 1;
  if (a != Dd - 1 && b != Dd - 1 && c != Dd - 1) return -1;
  if (nodes.x[0] != 0.0 || nodes.x[Dd - 1] != 1.0) return -1;
  const double h = leaf_side(g);
  double x = g.x + h * nodes.x[a], y = g.y + h * nodes.x[b], z = g.z + h * nodes.x[c];
  if (per) {
    x = wrap1(x);
    y = wrap1(y);
    z = wrap1(z);
  }
  if (!inside(x, y, z, per)) return -1;
  const int64_t B = find_leaf(dst, morton3(quantise(x), quantise(y), quantise(z)));
  if (B == leaf) return -1;
  const Geom gb = load_geom(dst.geom + B);
  if (gb.w != g.w) return -1;
  int ia = a, ib = b, ic = c;
  if (a == Dd - 1) {
    if (gb.x != x) return -1;
    ia = 0;
  } else if (gb.x != g.x) {
    return -1;
  }
  if (b == Dd - 1) {
    if (gb.y != y) return -1;
    ib = 0;
  } else if (gb.y != g.y) {
    return -1;
  }
  if (c == Dd - 1) {
    if (gb.z != z) return -1;
    ic = 0;
  } else if (gb.z != g.z) {
    return -1;
  }
  return B * (int64_t)Dd * Dd * Dd + ia + Dd * (ib + Dd * ic);
}

// Walks the destination leaf's nodes source leaf by source leaf.  Leaves
// tile the unit cube (tree_create checks it), so the nodes a source leaf
// holds are those inside its box: starting from the first node not yet
// visited, one key search finds its source leaf and per-axis box tests give
// the sub-grid.  outside(p) is called for nodes outside the domain, fn(sub)
// for every sub-grid (all threads, block-synchronised around it); with a face
// map (k_face_map's output, else null), nodes it maps to a neighbour's node
// are skipped.  The walk's shared memory is the first walk_smem(Ds, Dd)
// bytes of sm.
template <int Ds, class Outside, class Fn>
__device__ __forceinline__ void for_each_subgrid(const TreeView& S, const TreeView& dst,
                                                 const Nodes1D& nodes, bool per, int64_t leaf,
                                                 const int32_t* __restrict__ face, double* sm,
                                                 Outside outside, Fn fn) {
  __shared__ int s_first;
  __shared__ int s_n[3];
  const int Dd = dst.q + 1, Dd2 = Dd * Dd, Dd3 = Dd2 * Dd;
  const int tid = threadIdx.x, bs = blockDim.x;
  double* sx = sm;                                              // [3][Dd]
  double* sT = sx + 3 * Dd;                                     // [3][Ds][Dd]
  uint32_t* sq = reinterpret_cast<uint32_t*>(sT + 3 * Ds * Dd);  // [3][Dd] keys, ~0 outside
  int* sidx = reinterpret_cast<int*>(sq + 3 * Dd);              // [3][Dd]
  uint8_t* sdone = reinterpret_cast<uint8_t*>(sidx + 3 * Dd);   // [Dd^3]

  const Geom g = load_geom(dst.geom + leaf);
  const double h = leaf_side(g);
  if (tid < 3 * Dd) {
    const int ax = tid / Dd, i = tid - ax * Dd;
    const double o = ax == 0 ? g.x : (ax == 1 ? g.y : g.z);
    double c = o + h * nodes.x[i];
    if (per) c = wrap1(c);
    sx[tid] = c;
    // the per-axis part of inside(); a point is inside iff all three are
    const bool in = per ? in_unit_open(c) : in_unit_closed(c);
    sq[tid] = in ? (uint32_t)quantise(c) : 0xffffffffu;
  }
  __syncthreads();
  const int32_t* lface = face ? face + leaf * Dd3 : nullptr;
  for (int p = tid; p < Dd3; p += bs) {
    const bool in = sq[p % Dd] != 0xffffffffu && sq[Dd + (p / Dd) % Dd] != 0xffffffffu &&
                    sq[2 * Dd + p / Dd2] != 0xffffffffu;
    // shared upper-face nodes are left to the face copy
    const bool skip = !in || (lface && __ldg(lface + p) >= 0);
    sdone[p] = skip ? 1 : 0;
    if (!in) outside(p);
  }
  __syncthreads();

  for (;;) {
    if (tid == 0) s_first = INT_MAX;
    __syncthreads();
    int first = INT_MAX;
    for (int p = tid; p < Dd3; p += bs)
      if (!sdone[p]) {
        first = p;
        break;
      }
    if (first != INT_MAX) atomicMin(&s_first, first);
    __syncthreads();
    const int p0 = s_first;
    if (p0 == INT_MAX) break;
    const int64_t V = find_leaf(S, morton3(sq[p0 % Dd], sq[Dd + (p0 / Dd) % Dd],
                                           sq[2 * Dd + p0 / Dd2]));
    const Geom vg = load_geom(S.geom + V);
    // the box of V in key units: anchor * 2^21, side 2^21 / 2^depth, from
    // the exponent of w = 2^(depth+1) (no FP64 division)
    const uint32_t side = 1u << (kKeyBits - ((int)(dbits(vg.w) >> 52) - 1024));
    if (tid < 3) {
      const double o = tid == 0 ? vg.x : (tid == 1 ? vg.y : vg.z);
      const uint32_t lo = (uint32_t)quantise(o);  // anchors are exact multiples of 2^-21
      int n = 0;
      for (int i = 0; i < Dd; ++i) {
        const uint32_t k = sq[tid * Dd + i];
        if (k != 0xffffffffu && k >= lo && k - lo < side) sidx[tid * Dd + n++] = i;
      }
      s_n[tid] = n;
    }
    __syncthreads();
    const int na = s_n[0], nb = s_n[1], nz = s_n[2];
    // T tables of the listed indices (local coordinate and recurrence of
    // eval_point)
    if (tid < 3 * Dd) {
      const int ax = tid / Dd, i = tid - ax * Dd;
      const int n = ax == 0 ? na : (ax == 1 ? nb : nz);
      if (i < n) {
        const double c = sx[ax * Dd + sidx[ax * Dd + i]];
        const double o = ax == 0 ? vg.x : (ax == 1 ? vg.y : vg.z);
        cheb_T_col<Ds>((c - o) * vg.w - 1.0, sT + ax * Ds * Dd + i, Dd);
      }
    }
    __syncthreads();
    fn(SubGrid{V, na, nb, nz, sidx, sT, sT + Ds * Dd, sT + 2 * Ds * Dd});
    for (int o = tid; o < nz * nb * na; o += bs) {
      const int ai = o % na, r = o / na, bi = r % nb, ci = r / nb;
      sdone[sidx[ai] + Dd * (sidx[Dd + bi] + Dd * sidx[2 * Dd + ci])] = 1;
    }
    __syncthreads();
  }
}

// One destination leaf (the whole CTA) of the evaluation.  out: the
// destination tree's [L * Dd^3][src.dof] array.
template <int Ds>
__device__ __forceinline__ void eval_on_nodes_leaf(const TreeView& S, const TreeView& dst,
                                                   const Nodes1D& nodes, bool per, int64_t leaf,
                                                   const int32_t* face,
                                                   double* __restrict__ out_all, double* sm) {
  const int Dd = dst.q + 1, Dd3 = Dd * Dd * Dd;
  const int dof = S.dof;
  double* sw = sm + walk_smem(Ds, Dd) / 8;  // [dof][pair(i,j)][Dd]
  double* out = out_all + leaf * (int64_t)Dd3 * dof;
  for_each_subgrid<Ds>(
      S, dst, nodes, per, leaf, face, sm,
      [&](int p) {
        for (int l = 0; l < dof; ++l) out[(int64_t)p * dof + l] = 0.0;
      },
      [&](const SubGrid& sg) { eval_subgrid<Ds>(S, sg, Dd, out, dof, 1, sw); });
}

// Several source trees of one leaf structure (the walk's source leaves are
// the same for all of them): tree t's values go to out_all + t * tstride,
// [dst.L * Dd^3][dof] each.  The sub-grid passes take `group` trees at a
// time (dof x group components, whose w tables fill the shared memory),
// each value as eval_on_nodes_leaf computes it.  s_coeff: the trees'
// coefficient arrays, in shared memory.
template <int Ds>
__device__ __forceinline__ void eval_on_nodes_set_leaf(const TreeView& S, const TreeView& dst,
                                                       const Nodes1D& nodes, bool per,
                                                       int64_t leaf, const int32_t* face,
                                                       const double* const* s_coeff, int ntrees,
                                                       int group, double* __restrict__ out_all,
                                                       int64_t tstride, double* sm) {
  constexpr int NCs = Ds * (Ds + 1) * (Ds + 2) / 6;
  const int Dd = dst.q + 1, Dd3 = Dd * Dd * Dd;
  const int dof = S.dof;
  const int64_t stride = S.stride;
  double* sw = sm + walk_smem(Ds, Dd) / 8;
  double* out = out_all + leaf * (int64_t)Dd3 * dof;
  for_each_subgrid<Ds>(
      S, dst, nodes, per, leaf, face, sm,
      [&](int p) {
        for (int t = 0; t < ntrees; ++t)
          for (int l = 0; l < dof; ++l) out[t * tstride + (int64_t)p * dof + l] = 0.0;
      },
      [&](const SubGrid& sg) {
        for (int t0 = 0; t0 < ntrees; t0 += group) {
          if (t0 > 0) __syncthreads();  // the previous group is done with sw
          const int nt = min(group, ntrees - t0);
          eval_subgrid_comps<Ds>(
              sg, Dd, nt * dof,
              [=](int c) {
                const int t = c / dof;
                return s_coeff[t0 + t] + sg.V * stride + (c - t * dof) * NCs;
              },
              [=](int c) {
                const int t = c / dof;
                return out + (t0 + t) * tstride + (c - t * dof);
              },
              dof, sw);
        }
      });
}

// The transposed map (adjoint of the evaluation): for one destination leaf,
// out[V * out_stride + l * Nc + n] += sum over its nodes p inside V of
// W[p][l] phi_n(X_p), the basis of V at the node -- the same passes in
// reverse (z, then y, then x), one FP64 atomic per coefficient and sub-grid.
// W: [dst.L * Dd^3][dof].
template <int Ds, class A>
__device__ __forceinline__ void scatter_on_nodes_leaf(const TreeView& S, const TreeView& dst,
                                                      const Nodes1D& nodes, bool per,
                                                      int64_t leaf, const double* __restrict__ W,
                                                      double* __restrict__ out,
                                                      int64_t out_stride, double* sm) {
  typedef typename A::T T;
  constexpr int NCs = Ds * (Ds + 1) * (Ds + 2) / 6, npair = Ds * (Ds + 1) / 2;
  const int Dd = dst.q + 1, Dd2 = Dd * Dd, Dd3 = Dd2 * Dd;
  const int dof = S.dof;
  const int tid = threadIdx.x, bs = blockDim.x;
  T* sTT = reinterpret_cast<T*>(sm + walk_smem(Ds, Dd) / 8);  // [3][Ds][Dd] T in A
  T* sW = sTT + 3 * Ds * Dd;  // [c'][b'][a'] weights of one component
  T* sH = sW + Dd3;           // [i][b'][a']
  T* sG = sH + Ds * Dd2;      // [pair(i,j)][a']
  const double* Wl = W + leaf * (int64_t)Dd3 * dof;
  for_each_subgrid<Ds>(
      S, dst, nodes, per, leaf, nullptr, sm, [](int) {},
      [&](const SubGrid& sg) {
        const int na = sg.na, nb = sg.nb, nz = sg.nz;
        const int* sidx = sg.sidx;
        double* oV = out + sg.V * out_stride;
        for (int o = tid; o < 3 * Ds * Dd; o += bs) sTT[o] = A::from(sg.Tx[o]);
        __syncthreads();
        const T* Tx = sTT;
        const T* Ty = sTT + Ds * Dd;
        const T* Tz = sTT + 2 * Ds * Dd;
        for (int l = 0; l < dof; ++l) {
          for (int o = tid; o < nz * nb * na; o += bs) {
            const int ai = o % na, r = o / na, bi = r % nb, ci = r / nb;
            const int p = sidx[ai] + Dd * (sidx[Dd + bi] + Dd * sidx[2 * Dd + ci]);
            sW[o] = A::from(__ldg(Wl + (int64_t)p * dof + l));
          }
          __syncthreads();
          // H(i, b', a') = sum_c' T_i(z_c') W(c', b', a')
          for (int o = tid; o < Ds * nb * na; o += bs) {
            const int ai = o % na, r = o / na, bi = r % nb, i = r / nb;
            T s = A::zero();
            for (int ci = 0; ci < nz; ++ci) A::mac(s, Tz[i * Dd + ci], sW[(ci * nb + bi) * na + ai]);
            sH[(i * nb + bi) * na + ai] = A::done(s);
          }
          __syncthreads();
          // G(pair(i,j), a') = sum_b' T_j(y_b') H(i, b', a')
          for (int o = tid; o < npair * na; o += bs) {
            const int ai = o % na, pr = o / na;
            int i = 0, rem = pr;
            while (rem >= Ds - i) {
              rem -= Ds - i;
              ++i;
            }
            const int j = rem;
            T s = A::zero();
            for (int bi = 0; bi < nb; ++bi) A::mac(s, Ty[j * Dd + bi], sH[(i * nb + bi) * na + ai]);
            sG[pr * na + ai] = A::done(s);
          }
          __syncthreads();
          // coefficient (i,j,k): sum_a' T_k(x_a') G(pair(i,j), a')
          for (int n = tid; n < NCs; n += bs) {
            int i = 0, rem = n;  // triangular index -> (i, j, k)
            while (rem >= (Ds - i) * (Ds - i + 1) / 2) {
              rem -= (Ds - i) * (Ds - i + 1) / 2;
              ++i;
            }
            int j = 0;
            while (rem >= Ds - i - j) {
              rem -= Ds - i - j;
              ++j;
            }
            const int k = rem;
            const int pr = i * Ds - (i * (i - 1)) / 2 + j;
            T s = A::zero();
            for (int ai = 0; ai < na; ++ai) A::mac(s, Tx[k * Dd + ai], sG[pr * na + ai]);
            const double v = A::value(s);
            if (v != 0.0) atomicAdd(oV + l * NCs + n, v);
          }
          __syncthreads();
        }
      });
}

// The face map of a destination tree: per node, face_source's target index
// for shared upper-face nodes, else -1.  One CTA per leaf.
__global__ void __launch_bounds__(kNodeEvalThreads) k_face_map(const TreeView dst,
                                                               const Nodes1D nodes, int periodic,
                                                               int32_t* __restrict__ face) {
  const int Dd = dst.q + 1, Dd2 = Dd * Dd, Dd3 = Dd2 * Dd;
  const int64_t leaf = blockIdx.x;
  const Geom g = load_geom(dst.geom + leaf);
  for (int p = threadIdx.x; p < Dd3; p += blockDim.x) {
    const int a = p % Dd, b = (p / Dd) % Dd, c = p / Dd2;
    const int64_t src = face_source(dst, nodes, periodic != 0, leaf, g, a, b, c);
    face[leaf * Dd3 + p] = (int32_t)src;
  }
}

// The values the walk left to copy: every shared upper-face node takes its
// neighbour's value (run after the evaluation; a source node is never itself
// a shared upper-face node, so the copies do not chain).
__global__ void __launch_bounds__(kNodeEvalThreads) k_copy_face_nodes(
    const int32_t* __restrict__ face, int64_t n, int dof, double* __restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t src = __ldg(face + t);
  if (src < 0) return;
  for (int l = 0; l < dof; ++l) out[t * dof + l] = out[(int64_t)src * dof + l];
}

template <int Ds>
__global__ void __launch_bounds__(kNodeEvalThreads) k_eval_on_nodes(const NodeEvalJob j,
                                                                    int periodic) {
  extern __shared__ __align__(16) double sm[];
  eval_on_nodes_leaf<Ds>(j.src, j.dst, j.nodes, periodic != 0, blockIdx.x, j.face, j.out, sm);
}

struct NodeEvalSet {
  NodeEvalJob j;  // j.src: the first tree (leaf structure, degree, dof)
  const double* coeff[kTvMaxTrees];
  int ntrees, group;
  int64_t tstride;
};

template <int Ds>
__global__ void __launch_bounds__(kNodeEvalThreads) k_eval_on_nodes_set(const NodeEvalSet a,
                                                                        int periodic) {
  extern __shared__ __align__(16) double sm[];
  __shared__ const double* s_coeff[kTvMaxTrees];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < kTvMaxTrees; ++k) s_coeff[k] = a.coeff[k];
  }
  __syncthreads();
  eval_on_nodes_set_leaf<Ds>(a.j.src, a.j.dst, a.j.nodes, periodic != 0, blockIdx.x, a.j.face,
                             s_coeff, a.ntrees, a.group, a.j.out, a.tstride, sm);
}

// Batched: one CTA per (job, destination leaf) item; the jobs of one launch
// share the source degree Ds.
template <int Ds>
__global__ void __launch_bounds__(kNodeEvalThreads) k_batch_eval_on_nodes(
    const NodeEvalJob* __restrict__ jobs, const NodeEvalItem* __restrict__ items, int periodic) {
  extern __shared__ __align__(16) double sm[];
  __shared__ NodeEvalJob sj;
  const NodeEvalItem it = items[blockIdx.x];
  if (threadIdx.x == 0) sj = jobs[it.job];
  __syncthreads();
  eval_on_nodes_leaf<Ds>(sj.src, sj.dst, sj.nodes, periodic != 0, it.leaf, sj.face, sj.out, sm);
}

template <int Ds, class A>
__global__ void __launch_bounds__(kNodeEvalThreads) k_scatter_on_nodes(const NodeEvalJob j,
                                                                       const double* W,
                                                                       int64_t out_stride,
                                                                       int periodic) {
  extern __shared__ __align__(16) double sm[];
  scatter_on_nodes_leaf<Ds, A>(j.src, j.dst, j.nodes, periodic != 0, blockIdx.x, W, j.out,
                               out_stride, sm);
}

constexpr int kMaxD = TBSLAS_MAX_DEGREE + 1;

// Raise a kernel's dynamic shared-memory limit to its largest launch, once
// per device.
void allow_smem(const void* kernel, size_t bytes, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (!(done.load() & bit)) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    done.fetch_or(bit);
  }
}

template <int Ds>
void launch_single(const NodeEvalJob& j, int64_t L, int periodic, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  allow_smem((const void*)k_eval_on_nodes<Ds>, node_eval_smem(Ds, kMaxD, 3), done);
  k_eval_on_nodes<Ds><<<(unsigned)L, kNodeEvalThreads,
                        node_eval_smem(Ds, j.dst.q + 1, j.src.dof), s>>>(j, periodic);
}

// Shared memory of a set launch: the walk and `group` trees' w tables,
// the largest group up to kSetSmem (at least one tree).
constexpr size_t kSetSmem = 100 * 1024;
template <int Ds>
void launch_set(NodeEvalSet a, int64_t L, int periodic, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  const int Dd = a.j.dst.q + 1, dof = a.j.src.dof;
  const size_t walk = walk_smem(Ds, Dd), per_tree = (size_t)dof * Ds * (Ds + 1) / 2 * Dd * 8;
  int g = a.ntrees;
  while (g > 1 && walk + g * per_tree > kSetSmem) --g;
  a.group = g;
  const size_t bytes = walk + g * per_tree;
  // a group's bytes stay within kSetSmem, one tree's within the single
  // launch's largest
  allow_smem((const void*)k_eval_on_nodes_set<Ds>, std::max(kSetSmem, node_eval_smem(Ds, kMaxD, 3)),
             done);
  k_eval_on_nodes_set<Ds><<<(unsigned)L, kNodeEvalThreads, bytes, s>>>(a, periodic);
}

template <int Ds>
void launch_batched(const NodeEvalJob* jobs, const NodeEvalItem* items, int64_t n, int max_qd,
                    int periodic, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  allow_smem((const void*)k_batch_eval_on_nodes<Ds>, node_eval_smem(Ds, kMaxD, 3), done);
  k_batch_eval_on_nodes<Ds><<<(unsigned)n, kNodeEvalThreads, node_eval_smem(Ds, max_qd + 1, 3),
                              s>>>(jobs, items, periodic);
}

template <int Ds, class A>
void launch_scatter(const NodeEvalJob& j, const double* W, int64_t out_stride, int64_t L,
                    int periodic, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  allow_smem((const void*)k_scatter_on_nodes<Ds, A>, node_scatter_smem(Ds, kMaxD, 3), done);
  k_scatter_on_nodes<Ds, A><<<(unsigned)L, kNodeEvalThreads,
                              node_scatter_smem(Ds, j.dst.q + 1, j.src.dof), s>>>(j, W, out_stride,
                                                                                  periodic);
}

template <int Ds>
void dispatch_scatter(int ds, const NodeEvalJob& j, const double* W, int64_t out_stride,
                      int64_t L, int periodic, bool df_sums, cudaStream_t s) {
  if constexpr (Ds <= kMaxD) {
    if (ds == Ds) {
      if (df_sums)
        launch_scatter<Ds, NodeDF>(j, W, out_stride, L, periodic, s);
      else
        launch_scatter<Ds, NodeF64>(j, W, out_stride, L, periodic, s);
    } else {
      dispatch_scatter<Ds + 1>(ds, j, W, out_stride, L, periodic, df_sums, s);
    }
  }
}

template <int Ds>
void dispatch_single(int ds, const NodeEvalJob& j, int64_t L, int periodic, cudaStream_t s) {
  if constexpr (Ds <= kMaxD) {
    if (ds == Ds)
      launch_single<Ds>(j, L, periodic, s);
    else
      dispatch_single<Ds + 1>(ds, j, L, periodic, s);
  }
}

template <int Ds>
void dispatch_set(int ds, const NodeEvalSet& a, int64_t L, int periodic, cudaStream_t s) {
  if constexpr (Ds <= kMaxD) {
    if (ds == Ds)
      launch_set<Ds>(a, L, periodic, s);
    else
      dispatch_set<Ds + 1>(ds, a, L, periodic, s);
  }
}

template <int Ds>
void dispatch_batched(int ds, const NodeEvalJob* jobs, const NodeEvalItem* items, int64_t n,
                      int max_qd, int periodic, cudaStream_t s) {
  if constexpr (Ds <= kMaxD) {
    if (ds == Ds)
      launch_batched<Ds>(jobs, items, n, max_qd, periodic, s);
    else
      dispatch_batched<Ds + 1>(ds, jobs, items, n, max_qd, periodic, s);
  }
}

}  // namespace

void launch_face_map(const TreeView& dst, int periodic, int32_t* face, cudaStream_t s) {
  if (dst.L <= 0) return;
  Nodes1D nodes;
  std::memset(&nodes, 0, sizeof(nodes));
  const std::vector<double> x = cheb_nodes_1d(dst.q);
  for (int i = 0; i <= dst.q; ++i) nodes.x[i] = x[i];
  k_face_map<<<(unsigned)dst.L, kNodeEvalThreads, 0, s>>>(dst, nodes, periodic, face);
}

void launch_eval_on_nodes(const TreeView& src, const TreeView& dst, int periodic, double* out,
                          cudaStream_t s, const int32_t* face, bool copy_faces) {
  if (dst.L <= 0) return;
  NodeEvalJob j;
  j.src = src;
  j.dst = dst;
  std::memset(&j.nodes, 0, sizeof(j.nodes));
  const std::vector<double> x = cheb_nodes_1d(dst.q);
  for (int i = 0; i <= dst.q; ++i) j.nodes.x[i] = x[i];
  j.out = out;
  j.face = face;
  dispatch_single<1>(src.q + 1, j, dst.L, periodic, s);
  if (face && copy_faces) {
    const int64_t n = dst.L * (int64_t)(dst.q + 1) * (dst.q + 1) * (dst.q + 1);
    k_copy_face_nodes<<<(unsigned)((n + kNodeEvalThreads - 1) / kNodeEvalThreads),
                        kNodeEvalThreads, 0, s>>>(face, n, src.dof, out);
  }
}

void launch_eval_on_nodes_set(const TreeView* src, int ntrees, const TreeView& dst, int periodic,
                              double* out, int64_t tstride, cudaStream_t s,
                              const int32_t* face) {
  if (dst.L <= 0 || ntrees <= 0) return;
  NodeEvalSet a;
  std::memset(&a, 0, sizeof(a));
  a.j.src = src[0];
  a.j.dst = dst;
  const std::vector<double> x = cheb_nodes_1d(dst.q);
  for (int i = 0; i <= dst.q; ++i) a.j.nodes.x[i] = x[i];
  a.j.out = out;
  a.j.face = face;
  for (int k = 0; k < ntrees; ++k) a.coeff[k] = src[k].coeff;
  a.ntrees = ntrees;
  a.tstride = tstride;
  dispatch_set<1>(src[0].q + 1, a, dst.L, periodic, s);
}

void launch_scatter_on_nodes(const TreeView& src, const TreeView& dst, int periodic,
                             const double* W, double* out, int64_t out_stride, bool df_sums,
                             cudaStream_t s) {
  if (dst.L <= 0) return;
  NodeEvalJob j;
  j.src = src;
  j.dst = dst;
  std::memset(&j.nodes, 0, sizeof(j.nodes));
  const std::vector<double> x = cheb_nodes_1d(dst.q);
  for (int i = 0; i <= dst.q; ++i) j.nodes.x[i] = x[i];
  j.out = out;
  j.face = nullptr;
  dispatch_scatter<1>(src.q + 1, j, W, out_stride, dst.L, periodic, df_sums, s);
}

void launch_batch_eval_on_nodes(const NodeEvalJob* jobs, const NodeEvalItem* items,
                                int64_t n_items, int q_src, int max_q_dst, int periodic,
                                cudaStream_t s) {
  if (n_items <= 0) return;
  dispatch_batched<1>(q_src + 1, jobs, items, n_items, max_q_dst, periodic, s);
}

}  // namespace tbg
