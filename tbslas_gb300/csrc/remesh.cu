// Kernels of the adaptive re-meshing after a step (the reference's
// tcon.RefineTree(); tcon.Balance21(bc), src/applications/src/advection.cpp:
// 305-311; the rules live in PVFMM, not vendored -- this is the project's
// restatement, see tbslas_tree_remesh):
//   k_leaf_tails      tail = sum over dofs of |c| over the total-degree-q terms
//   k_sibling_groups  first leaf of every complete group of 8 siblings
//   k_transfer<D>     node values of new leaves from old ones: a child from
//                     its parent's expansion (restriction), a parent from its
//                     8 children (each node from the child whose closed half
//                     holds it), by the sum-factorised passes of the node grid
//   k_rebuild         the new leaf list from per-leaf actions (keep, split,
//                     merge) and exclusive scans of their counts
//   k_place_coeffs    coefficients of the new leaves (copied bit for bit, or
//                     from the transfer's refit)
//   k_balance_flags   leaves with a neighbour more than one level deeper
//   k_build_table     the coarse lookup table of find_leaf
// The host sequence is tree_remesh in capi.cu.
#include <atomic>
#include <cstring>
#include <vector>

#include "host_cheb.h"
#include "internal.h"
#include "node_passes.cuh"

namespace tbg {

namespace {

constexpr int kXferThreads = 256;

__device__ __forceinline__ int leaf_depth(const Geom& g) { return ilogb(g.w) - 1; }

// Shared memory of k_transfer at degree D (Ds = Dd = D): node coordinates
// [3][D], T tables [3][D][D], index lists [3][D] (ints, padded to 8 bytes),
// the first pass's buffer [dof][D(D+1)/2][D].
__host__ __device__ constexpr size_t xfer_smem(int D, int dof) {
  return (size_t)(3 * D + 3 * D * D) * 8 + (size_t)((3 * D + 1) / 2) * 8 +
         (size_t)dof * D * (D + 1) / 2 * D * 8;
}

template <int D>
__global__ void __launch_bounds__(kXferThreads) k_transfer(const TreeView S,
                                                           const XferItem* __restrict__ items,
                                                           const Nodes1D nodes,
                                                           double* __restrict__ out) {
  extern __shared__ __align__(16) double sm[];
  double* sx = sm;                                        // [3][D]
  double* sT = sx + 3 * D;                                // [3][D][D]
  int* sidx = reinterpret_cast<int*>(sT + 3 * D * D);     // [3][D]
  double* sw = reinterpret_cast<double*>(sidx) + (3 * D + 1) / 2;
  const XferItem it = items[blockIdx.x];
  const int tid = threadIdx.x;
  const double h = 2.0 / it.g.w;
  if (tid < 3 * D) {
    const int ax = tid / D, i = tid - ax * D;
    const double o = ax == 0 ? it.g.x : (ax == 1 ? it.g.y : it.g.z);
    sx[tid] = o + h * nodes.x[i];
  }
  const bool parent = it.mode == kXferParent;
  int m = D;  // nodes below the middle of the parent go to the lower child
  if (parent) {
    m = 0;
    while (m < D && nodes.x[m] < 0.5) ++m;
  }
  double* o_leaf = out + (int64_t)blockIdx.x * S.dof * D * D * D;
  const int nsub = parent ? 8 : 1;
  for (int c = 0; c < nsub; ++c) {
    int lo[3], n[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const int bit = (c >> ax) & 1;
      lo[ax] = parent ? (bit ? m : 0) : 0;
      n[ax] = parent ? (bit ? D - m : m) : D;
    }
    const int64_t V = it.src + (parent ? c : 0);
    __syncthreads();  // the previous sub-grid is done with sidx and sT
    const Geom vg = load_geom(S.geom + V);
    if (tid < 3 * D) {
      const int ax = tid / D, i = tid - ax * D;
      if (i < n[ax]) {
        const double o = ax == 0 ? vg.x : (ax == 1 ? vg.y : vg.z);
        sidx[ax * D + i] = lo[ax] + i;
        cheb_T_col<D>((sx[ax * D + lo[ax] + i] - o) * vg.w - 1.0, sT + ax * D * D + i, D);
      }
    }
    __syncthreads();
    if (n[0] > 0 && n[1] > 0 && n[2] > 0)
      eval_subgrid<D>(S, SubGrid{V, n[0], n[1], n[2], sidx, sT, sT + D * D, sT + 2 * D * D}, D,
                      o_leaf, 1, (int64_t)D * D * D, sw);
  }
}

__global__ void k_leaf_tails(const double* __restrict__ coeff, int64_t L, int dof, int q,
                             int64_t stride, double* __restrict__ tail) {
  const int64_t leaf = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (leaf >= L) return;
  const int D = q + 1, NC = D * (D + 1) * (D + 2) / 6;
  double s = 0.0;
  for (int l = 0; l < dof; ++l) {
    const double* c = coeff + leaf * stride + (int64_t)l * NC;
    int idx = 0;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D - i; ++j) {
        idx += D - i - j;
        s += fabs(c[idx - 1]);  // k = q - i - j: the row's last term
      }
  }
  tail[leaf] = s;
}

__global__ void k_sibling_groups(const uint64_t* __restrict__ keys, const Geom* __restrict__ geom,
                                 int64_t L, int min_depth, int64_t* __restrict__ first) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L) return;
  int64_t f = 0;
  const int d = leaf_depth(geom[i]);
  if (d > min_depth && i + 7 < L) {
    const uint64_t unit = 1ull << (3 * (kKeyBits - d));
    if (keys[i] % (8 * unit) == 0 && keys[i + 7] == keys[i] + 7 * unit &&
        leaf_depth(geom[i + 7]) == d)
      f = 1;
  }
  first[i] = f;
}

// Group g (first leaf i): the parent's transfer item.
__global__ void k_group_items(const int64_t* __restrict__ first, const int64_t* __restrict__ pos,
                              const Geom* __restrict__ geom, int64_t L,
                              XferItem* __restrict__ items, int64_t* __restrict__ group_leaf) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L || !first[i]) return;
  const int64_t g = pos[i];
  Geom p = geom[i];
  p.w *= 0.5;
  items[g] = XferItem{p, i, kXferParent, 0};
  group_leaf[g] = i;
}

// Merge decisions: the 8 leaves of group g become its parent when tail <= tol.
__global__ void k_merge_actions(const int64_t* __restrict__ group_leaf, int64_t G,
                                const double* __restrict__ tail, double tol,
                                int8_t* __restrict__ act, int64_t* __restrict__ aux) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= G || !(tail[g] <= tol)) return;
  const int64_t i = group_leaf[g];
  act[i] = kActMerge;
  aux[i] = g;
  for (int c = 1; c < 8; ++c) act[i + c] = kActDrop;
}

__global__ void k_split_actions(const double* __restrict__ tail, const Geom* __restrict__ geom,
                                int64_t L, double tol, int max_depth, int8_t* __restrict__ act,
                                unsigned long long* __restrict__ count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L) return;
  const bool split = tail[i] > tol && leaf_depth(geom[i]) < max_depth;
  act[i] = split ? kActSplit : kActKeep;
  if (split) atomicAdd(count, 1ull);
}

// New leaves per action (keep 1, split 8, merge 1, drop 0) and transfer items
// per action (split 8).
__global__ void k_action_counts(const int8_t* __restrict__ act, int64_t L,
                                int64_t* __restrict__ nleaf, int64_t* __restrict__ nxfer) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L) return;
  const int a = act[i];
  nleaf[i] = a == kActSplit ? 8 : (a == kActDrop ? 0 : 1);
  nxfer[i] = a == kActSplit ? 8 : 0;
}

// src_of[new leaf]: >= 0 old leaf to copy; -(1 + k) compact coefficient row k
// of the merge buffer (kind 1) or of the split buffer (kind 2), encoded as
// kind * 2^40 + k.
__global__ void k_rebuild(const uint64_t* __restrict__ keys, const Geom* __restrict__ geom,
                          const int8_t* __restrict__ act, const int64_t* __restrict__ aux,
                          const int64_t* __restrict__ pos, const int64_t* __restrict__ xpos,
                          int64_t L, uint64_t* __restrict__ nkeys, Geom* __restrict__ ngeom,
                          int64_t* __restrict__ src_of, XferItem* __restrict__ items) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L) return;
  const int a = act[i];
  const int64_t p = pos[i];
  const Geom g = geom[i];
  if (a == kActKeep) {
    nkeys[p] = keys[i];
    ngeom[p] = g;
    src_of[p] = i;
  } else if (a == kActMerge) {
    Geom pg = g;
    pg.w *= 0.5;
    nkeys[p] = keys[i];
    ngeom[p] = pg;
    src_of[p] = -(1 + ((int64_t)1 << 40) + aux[i]);
  } else if (a == kActSplit) {
    const double hc = 1.0 / g.w;  // half the leaf's side
    const int d = leaf_depth(g) + 1;
    const uint64_t unit = 1ull << (3 * (kKeyBits - d));
    for (int c = 0; c < 8; ++c) {
      Geom cg{g.x + ((c & 1) ? hc : 0.0), g.y + ((c & 2) ? hc : 0.0), g.z + ((c & 4) ? hc : 0.0),
              2.0 * g.w};
      nkeys[p + c] = keys[i] + (uint64_t)c * unit;
      ngeom[p + c] = cg;
      const int64_t k = xpos[i] + c;
      src_of[p + c] = -(1 + ((int64_t)2 << 40) + k);
      items[k] = XferItem{cg, i, kXferChild, 0};
    }
  }
}

// One CTA per new leaf: its stride coefficients.
__global__ void k_place_coeffs(const int64_t* __restrict__ src_of, int64_t stride,
                               const double* __restrict__ old_c, const double* __restrict__ merge_c,
                               const double* __restrict__ split_c, double* __restrict__ out) {
  const int64_t leaf = blockIdx.x;
  const int64_t s = src_of[leaf];
  const double* src;
  if (s >= 0) {
    src = old_c + s * stride;
  } else {
    const int64_t e = -s - 1;
    const int64_t kind = e >> 40, k = e & (((int64_t)1 << 40) - 1);
    src = (kind == 1 ? merge_c : split_c) + k * stride;
  }
  for (int64_t t = threadIdx.x; t < stride; t += blockDim.x) out[leaf * stride + t] = src[t];
}

// Leaves with a face, edge or corner neighbour more than one level deeper:
// each of the 26 probes lies half a key unit outside the leaf's box.
__global__ void k_balance_flags(const TreeView t, int periodic, int8_t* __restrict__ act,
                                unsigned long long* __restrict__ count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= t.L) return;
  const Geom g = t.geom[i];
  const int d = leaf_depth(g);
  const double h = leaf_side(g);
  const double cx = g.x + 0.5 * h, cy = g.y + 0.5 * h, cz = g.z + 0.5 * h;
  const double r = 0.5 * h + 0x1p-22;
  bool split = false;
  for (int n = 0; n < 27 && !split; ++n) {
    if (n == 13) continue;
    double p[3] = {cx + (double)(n % 3 - 1) * r, cy + (double)((n / 3) % 3 - 1) * r,
                   cz + (double)(n / 9 - 1) * r};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (periodic) {
        p[a] = wrap1(p[a]);
      } else if (!(p[a] >= 0.0 && p[a] < 1.0)) {
        ok = false;
      }
    }
    if (!ok) continue;
    const int64_t nb = find_leaf(t, morton3(quantise(p[0]), quantise(p[1]), quantise(p[2])));
    if (leaf_depth(t.geom[nb]) > d + 1) split = true;
  }
  act[i] = split ? kActSplit : kActKeep;
  if (split) atomicAdd(count, 1ull);
}

__global__ void k_build_table(const uint64_t* __restrict__ keys, int64_t L, int T,
                              int32_t* __restrict__ table) {
  const int64_t ncell = 1ll << (3 * T);
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c > ncell) return;
  if (c == ncell) {
    table[c] = (int32_t)(L - 1);
    return;
  }
  const uint64_t ck = (uint64_t)c << (3 * (kKeyBits - T));
  int64_t lo = 0, hi = L - 1;  // last leaf with key <= ck (keys[0] == 0)
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (keys[mid] <= ck) lo = mid; else hi = mid - 1;
  }
  table[c] = (int32_t)lo;
}

__global__ void k_max_depth(const Geom* __restrict__ geom, int64_t L, int* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < L) atomicMax(out, leaf_depth(geom[i]));
}

inline unsigned blocks_of(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <int D>
void launch_transfer_d(const TreeView& S, const XferItem* items, int64_t n, const Nodes1D& nodes,
                       double* out, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const size_t smem = xfer_smem(D, S.dof);
  const uint64_t bit = 1ull << (dev & 63);
  if (!(done.load() & bit)) {
    cudaFuncSetAttribute(k_transfer<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)xfer_smem(D, 3));
    done.fetch_or(bit);
  }
  k_transfer<D><<<(unsigned)n, kXferThreads, smem, s>>>(S, items, nodes, out);
}

template <int D>
void dispatch_transfer(int d, const TreeView& S, const XferItem* items, int64_t n,
                       const Nodes1D& nodes, double* out, cudaStream_t s) {
  if constexpr (D <= TBSLAS_MAX_DEGREE + 1) {
    if (d == D)
      launch_transfer_d<D>(S, items, n, nodes, out, s);
    else
      dispatch_transfer<D + 1>(d, S, items, n, nodes, out, s);
  }
}

}  // namespace

void launch_transfer(const TreeView& S, const XferItem* items, int64_t n, const Nodes1D& nodes,
                     double* out, cudaStream_t s) {
  if (n > 0) dispatch_transfer<2>(S.q + 1, S, items, n, nodes, out, s);
}

void launch_leaf_tails(const double* coeff, int64_t L, int dof, int q, int64_t stride,
                       double* tail, cudaStream_t s) {
  if (L > 0) k_leaf_tails<<<blocks_of(L, 128), 128, 0, s>>>(coeff, L, dof, q, stride, tail);
}

void launch_sibling_groups(const uint64_t* keys, const Geom* geom, int64_t L, int min_depth,
                           int64_t* first, cudaStream_t s) {
  if (L > 0) k_sibling_groups<<<blocks_of(L, 256), 256, 0, s>>>(keys, geom, L, min_depth, first);
}

void launch_group_items(const int64_t* first, const int64_t* pos, const Geom* geom, int64_t L,
                        XferItem* items, int64_t* group_leaf, cudaStream_t s) {
  if (L > 0)
    k_group_items<<<blocks_of(L, 256), 256, 0, s>>>(first, pos, geom, L, items, group_leaf);
}

void launch_merge_actions(const int64_t* group_leaf, int64_t G, const double* tail, double tol,
                          int8_t* act, int64_t* aux, cudaStream_t s) {
  if (G > 0)
    k_merge_actions<<<blocks_of(G, 256), 256, 0, s>>>(group_leaf, G, tail, tol, act, aux);
}

void launch_split_actions(const double* tail, const Geom* geom, int64_t L, double tol,
                          int max_depth, int8_t* act, unsigned long long* count, cudaStream_t s) {
  if (L > 0)
    k_split_actions<<<blocks_of(L, 256), 256, 0, s>>>(tail, geom, L, tol, max_depth, act, count);
}

void launch_action_counts(const int8_t* act, int64_t L, int64_t* nleaf, int64_t* nxfer,
                          cudaStream_t s) {
  if (L > 0) k_action_counts<<<blocks_of(L, 256), 256, 0, s>>>(act, L, nleaf, nxfer);
}

void launch_rebuild(const uint64_t* keys, const Geom* geom, const int8_t* act, const int64_t* aux,
                    const int64_t* pos, const int64_t* xpos, int64_t L, uint64_t* nkeys,
                    Geom* ngeom, int64_t* src_of, XferItem* items, cudaStream_t s) {
  if (L > 0)
    k_rebuild<<<blocks_of(L, 256), 256, 0, s>>>(keys, geom, act, aux, pos, xpos, L, nkeys, ngeom,
                                                src_of, items);
}

void launch_place_coeffs(const int64_t* src_of, int64_t Lnew, int64_t stride, const double* old_c,
                         const double* merge_c, const double* split_c, double* out,
                         cudaStream_t s) {
  if (Lnew > 0)
    k_place_coeffs<<<(unsigned)Lnew, 128, 0, s>>>(src_of, stride, old_c, merge_c, split_c, out);
}

void launch_balance_flags(const TreeView& t, int periodic, int8_t* act, unsigned long long* count,
                          cudaStream_t s) {
  if (t.L > 0) k_balance_flags<<<blocks_of(t.L, 128), 128, 0, s>>>(t, periodic, act, count);
}

void launch_build_table(const uint64_t* keys, int64_t L, int T, int32_t* table, cudaStream_t s) {
  const int64_t n = (1ll << (3 * T)) + 1;
  k_build_table<<<blocks_of(n, 256), 256, 0, s>>>(keys, L, T, table);
}

void launch_max_depth(const Geom* geom, int64_t L, int* out, cudaStream_t s) {
  if (L > 0) k_max_depth<<<blocks_of(L, 256), 256, 0, s>>>(geom, L, out);
}

}  // namespace tbg
