// Node values -> Chebyshev coefficients of every leaf (SetTreeGridValues,
// src/tree/tree_utils.h:500-552), which the reference computes as one dense
// product with the Np x Nc matrix M = pinv(V)^T (GetPt2CoeffMatrix,
// src/utils/cheb.h:166-196).  The same linear map factors through the 1-D
// QR A = Q R of the Chebyshev-Vandermonde matrix at the stretched nodes
// (refit_factors, host_cheb.cpp):
//   c = [ (R^-1)^(x)3 ext_T( [ (Q^T)^(x)3 f ]_T ) ]_T ,  T = {i+j+k < D},
// three 1-D passes with Q^T over the box (D^4 + D^4/2 + D^4/6 multiply-adds)
// and three triangular passes with R^-1 inside T (~D^4/24 each): ~1.8 D^4
// per leaf and component instead of D^3 Nc (D^6/6) -- 25x fewer at q = 14.
// One CTA per (leaf, component) row; the row and its intermediates live in
// shared memory (two D^3 buffers).  The passes run in FP64 or, for the
// double-float step, in double-float on the FP32 pipe.
#include <atomic>

#include "internal.h"

namespace tbg {

namespace {

constexpr int kRefitThreads = 256;

__host__ __device__ constexpr int nc_of(int n) { return n * (n + 1) * (n + 2) / 6; }

// Position of coefficient (i, j, k) (z, y, x degrees) in the triangular order
// i outer, j, k inner.
__device__ __forceinline__ int tri_index(int D, int i, int j, int k) {
  const int m = D - i;
  return nc_of(D) - nc_of(m) + j * m - (j * (j - 1)) / 2 + k;
}

// Arithmetic of the passes: FP64, or double-float (df64.cuh) -- a value is a
// float2 hi/lo pair, every dot product is accumulated with the error-free
// df_fma_acc and renormalised (~1e-15 relative per pass, on the FP32 pipe).
struct ArithF64 {
  typedef double T;
  __device__ static T zero() { return 0.0; }
  __device__ static void mac(T& acc, T a, T b) { acc = fma(a, b, acc); }
  __device__ static T done(T acc) { return acc; }
  __device__ static T from(double x) { return x; }
  __device__ static double value(T v) { return v; }
};
struct ArithDF {
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
  __device__ static double value(T v) { return df_to_double(df{v.x, v.y}); }
};

template <class A>
struct Factors {  // shared-memory views of the 4 D x D blocks
  const typename A::T *Q, *QT, *Ri, *RiT;
};

template <class A>
__device__ __forceinline__ Factors<A> stage_factors(const double* __restrict__ F, int D,
                                                    typename A::T* sm) {
  const int n = 4 * D * D;
  for (int e = threadIdx.x; e < n; e += blockDim.x) sm[e] = A::from(__ldg(F + e));
  const int dd = D * D;
  return Factors<A>{sm, sm + dd, sm + 2 * dd, sm + 3 * dd};
}

// Box positions of the triangle T and of its (j, k) pairs, so that the passes
// inside T run over compact lists (every lane of a warp busy) rather than
// over the box with most lanes masked:
//   tri[n]  = i D^2 + j D + k of triangular index n (i outer, j, k inner),
//   pair[n] = j D + k of the n-th pair with j + k < D (j outer).
// Built by the block; followed by a barrier.
struct TriLists {
  const int* tri;
  const int* pair;
};
__device__ __forceinline__ TriLists build_tri_lists(int D, int* tri, int* pair) {
  const int D2 = D * D, NC = nc_of(D), NP = D * (D + 1) / 2;
  for (int n = threadIdx.x; n < NC; n += blockDim.x) {
    int i = 0, rem = n;
    while (rem >= (D - i) * (D - i + 1) / 2) {
      rem -= (D - i) * (D - i + 1) / 2;
      ++i;
    }
    int j = 0;
    while (rem >= D - i - j) {
      rem -= D - i - j;
      ++j;
    }
    tri[n] = i * D2 + j * D + rem;
  }
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    int j = 0, rem = n;
    while (rem >= D - j) {
      rem -= D - j;
      ++j;
    }
    pair[n] = j * D + rem;
  }
  __syncthreads();
  return TriLists{tri, pair};
}

// f (D^3 values, x fastest) in S0 -> coefficients, handed to `emit(t, c)`
// with t the triangular index (FP64).  Ends with the block synchronised.
// Every output is one thread's dot product in a fixed order, so the result
// does not depend on which thread computes it.
template <class A, class Emit>
__device__ __forceinline__ void refit_row(const Factors<A>& f, const TriLists& tl, int D,
                                          typename A::T* S0, typename A::T* S1, Emit emit) {
  typedef typename A::T T;
  const int D2 = D * D, D3 = D2 * D, NC = nc_of(D), NP = D * (D + 1) / 2;
  const int tid = threadIdx.x, bs = blockDim.x;
  // x: S1[c][b][k] = sum_a Q[a][k] S0[c][b][a]
  for (int o = tid; o < D3; o += bs) {
    const int k = o % D;
    const T* row = S0 + (o - k);
    T s = A::zero();
    for (int a = 0; a < D; ++a) A::mac(s, f.Q[a * D + k], row[a]);
    S1[o] = A::done(s);
  }
  __syncthreads();
  // y: S0[c][j][k] = sum_b Q[b][j] S1[c][b][k],  j + k < D
  for (int m = tid; m < D * NP; m += bs) {
    const int c = m / NP, jk = tl.pair[m - c * NP];
    const int k = jk % D, j = jk / D;
    const T* col = S1 + c * D2 + k;
    T s = A::zero();
    for (int b = 0; b < D; ++b) A::mac(s, f.Q[b * D + j], col[b * D]);
    S0[c * D2 + jk] = A::done(s);
  }
  __syncthreads();
  // z: S1[i][j][k] = sum_c Q[c][i] S0[c][j][k],  i + j + k < D
  for (int m = tid; m < NC; m += bs) {
    const int o = tl.tri[m];
    const int k = o % D, j = (o / D) % D, i = o / D2;
    const T* col = S0 + j * D + k;
    T s = A::zero();
    for (int c = 0; c < D; ++c) A::mac(s, f.Q[c * D + i], col[c * D2]);
    S1[o] = A::done(s);
  }
  __syncthreads();
  // R^-1 along x: S0[i][j][k'] = sum_{k >= k'} R^-1[k'][k] S1[i][j][k]
  for (int m = tid; m < NC; m += bs) {
    const int o = tl.tri[m];
    const int k = o % D, j = (o / D) % D, i = o / D2;
    const int n = D - i - j;
    const T* row = S1 + (o - k);
    T s = A::zero();
    for (int kk = k; kk < n; ++kk) A::mac(s, f.RiT[kk * D + k], row[kk]);
    S0[o] = A::done(s);
  }
  __syncthreads();
  // R^-1 along y: S1[i][j'][k] = sum_{j >= j'} R^-1[j'][j] S0[i][j][k]
  for (int m = tid; m < NC; m += bs) {
    const int o = tl.tri[m];
    const int k = o % D, j = (o / D) % D, i = o / D2;
    const int n = D - i - k;
    const T* col = S0 + i * D2 + k;
    T s = A::zero();
    for (int jj = j; jj < n; ++jj) A::mac(s, f.Ri[j * D + jj], col[jj * D]);
    S1[o] = A::done(s);
  }
  __syncthreads();
  // R^-1 along z: c[i'][j][k] = sum_{i >= i'} R^-1[i'][i] S1[i][j][k]
  for (int m = tid; m < NC; m += bs) {
    const int o = tl.tri[m];
    const int k = o % D, j = (o / D) % D, i = o / D2;
    const int n = D - j - k;
    const T* col = S1 + j * D + k;
    T s = A::zero();
    for (int ii = i; ii < n; ++ii) A::mac(s, f.Ri[i * D + ii], col[ii * D2]);
    emit(m, A::value(A::done(s)));  // m is the triangular index of (i, j, k)
  }
  __syncthreads();
}

// The transposed map, f = M c (M: Np x Nc): c (triangular order) in S0 at
// the box positions of T ->
//   f = (Q)^(x)3 ext_T( [ (R^-T)^(x)3 c ]_T ),
// handed to `emit(p, value)` with p the node index (x fastest).
template <class A, class Emit>
__device__ __forceinline__ void refit_row_t(const Factors<A>& f, const TriLists& tl, int D,
                                            typename A::T* S0, typename A::T* S1, Emit emit) {
  typedef typename A::T T;
  const int D2 = D * D, D3 = D2 * D, NC = nc_of(D), NP = D * (D + 1) / 2;
  const int tid = threadIdx.x, bs = blockDim.x;
  // R^-T along z: S1[i][j][k] = sum_{i' <= i} R^-1[i'][i] S0[i'][j][k]
  for (int m = tid; m < NC; m += bs) {
    const int o = tl.tri[m];
    const int k = o % D, j = (o / D) % D, i = o / D2;
    const T* col = S0 + j * D + k;
    T s = A::zero();
    for (int ii = 0; ii <= i; ++ii) A::mac(s, f.RiT[i * D + ii], col[ii * D2]);
    S1[o] = A::done(s);
  }
  __syncthreads();
  // R^-T along y
  for (int m = tid; m < NC; m += bs) {
    const int o = tl.tri[m];
    const int k = o % D, j = (o / D) % D, i = o / D2;
    const T* col = S1 + i * D2 + k;
    T s = A::zero();
    for (int jj = 0; jj <= j; ++jj) A::mac(s, f.RiT[j * D + jj], col[jj * D]);
    S0[o] = A::done(s);
  }
  __syncthreads();
  // R^-T along x
  for (int m = tid; m < NC; m += bs) {
    const int o = tl.tri[m];
    const int k = o % D;
    const T* row = S0 + (o - k);
    T s = A::zero();
    for (int kk = 0; kk <= k; ++kk) A::mac(s, f.Ri[kk * D + k], row[kk]);
    S1[o] = A::done(s);
  }
  __syncthreads();
  // Q along z: S0[c][j][k] = sum_{i < D-j-k} Q[c][i] S1[i][j][k],  j + k < D
  for (int m = tid; m < D * NP; m += bs) {
    const int c = m / NP, jk = tl.pair[m - c * NP];
    const int k = jk % D, j = jk / D;
    const int n = D - j - k;
    const T* col = S1 + j * D + k;
    T s = A::zero();
    for (int i = 0; i < n; ++i) A::mac(s, f.Q[c * D + i], col[i * D2]);
    S0[c * D2 + jk] = A::done(s);
  }
  __syncthreads();
  // Q along y: S1[c][b][k] = sum_{j < D-k} Q[b][j] S0[c][j][k]
  for (int o = tid; o < D3; o += bs) {
    const int k = o % D, b = (o / D) % D, c = o / D2;
    const int n = D - k;
    const T* col = S0 + c * D2 + k;
    T s = A::zero();
    for (int j = 0; j < n; ++j) A::mac(s, f.Q[b * D + j], col[j * D]);
    S1[o] = A::done(s);
  }
  __syncthreads();
  // Q along x: f[c][b][a] = sum_k Q[a][k] S1[c][b][k]
  for (int o = tid; o < D3; o += bs) {
    const int a = o % D;
    const T* row = S1 + (o - a);
    T s = A::zero();
    for (int k = 0; k < D; ++k) A::mac(s, f.QT[k * D + a], row[k]);
    emit(o, A::value(A::done(s)));
  }
  __syncthreads();
}

template <class A>
__device__ __forceinline__ void load_row(const double* __restrict__ v, int n,
                                         typename A::T* S0) {
  for (int e = threadIdx.x; e < n; e += blockDim.x) S0[e] = A::from(__ldg(v + e));
  __syncthreads();
}

struct CoeffOut {
  double* c;
  float2* c2;
  uint32_t* err;
  __device__ __forceinline__ void operator()(int t, double s) const {
    c[t] = s;
    if (c2) {
      check_df_range(s, err);
      const df v = df_from_double(s);
      c2[t] = make_float2(v.hi, v.lo);
    }
  }
};

// Dynamic shared memory of the refit kernels at degree q.
__host__ __device__ constexpr size_t refit_smem(int q) {
  return (size_t)(4 * (q + 1) * (q + 1) + 2 * (q + 1) * (q + 1) * (q + 1)) * sizeof(double) +
         (size_t)(nc_of(q + 1) + (q + 1) * (q + 2) / 2) * sizeof(int);
}
// The triangle lists sit after the two D^3 buffers.
__device__ __forceinline__ TriLists tri_lists_at(void* after_buffers, int D) {
  int* tri = reinterpret_cast<int*>(after_buffers);
  return build_tri_lists(D, tri, tri + nc_of(D));
}

template <class A>
__global__ void __launch_bounds__(kRefitThreads) k_refit(const double* __restrict__ vals,
                                                         const double* __restrict__ F, int q,
                                                         int dof, int64_t stride,
                                                         double* __restrict__ coeff,
                                                         float2* __restrict__ coeff2,
                                                         uint32_t* err) {
  typedef typename A::T T;
  extern __shared__ __align__(16) double sm_raw[];
  T* sm = reinterpret_cast<T*>(sm_raw);
  const int D = q + 1, D3 = D * D * D;
  const Factors<A> f = stage_factors<A>(F, D, sm);
  T* S0 = sm + 4 * D * D;
  T* S1 = S0 + D3;
  const TriLists tl = tri_lists_at(S1 + D3, D);
  const int64_t r = blockIdx.x;
  const int64_t leaf = r / dof;
  const int l = (int)(r - leaf * dof);
  load_row<A>(vals + r * D3, D3, S0);
  const int64_t base = leaf * stride + (int64_t)l * nc_of(D);
  refit_row<A>(f, tl, D, S0, S1, CoeffOut{coeff + base, coeff2 ? coeff2 + base : nullptr, err});
}

// mu[r][p] = sum_n M[p][n] lam[r][n] (the adjoint's transposed refit).
template <class A>
__global__ void __launch_bounds__(kRefitThreads) k_refit_t(const double* __restrict__ lam,
                                                           const double* __restrict__ F, int q,
                                                           double* __restrict__ mu) {
  typedef typename A::T T;
  extern __shared__ __align__(16) double sm_raw[];
  T* sm = reinterpret_cast<T*>(sm_raw);
  const int D = q + 1, D2 = D * D, D3 = D2 * D, NC = nc_of(D);
  const Factors<A> f = stage_factors<A>(F, D, sm);
  T* S0 = sm + 4 * D2;
  T* S1 = S0 + D3;
  const TriLists tl = tri_lists_at(S1 + D3, D);
  const int64_t r = blockIdx.x;
  const double* c = lam + r * NC;
  for (int o = threadIdx.x; o < D3; o += blockDim.x) {
    const int k = o % D, j = (o / D) % D, i = o / D2;
    if (i + j + k < D) S0[o] = A::from(__ldg(c + tri_index(D, i, j, k)));
  }
  __syncthreads();
  double* out = mu + r * D3;
  refit_row_t<A>(f, tl, D, S0, S1, [out](int p, double v) { out[p] = v; });
}

// Batched refit: one CTA per (problem, row) item.
template <class A>
__global__ void __launch_bounds__(kRefitThreads) k_batch_refit(const RefitJob* __restrict__ jobs,
                                                               const RefitItem* __restrict__ items) {
  typedef typename A::T T;
  extern __shared__ __align__(16) double sm_raw[];
  T* sm = reinterpret_cast<T*>(sm_raw);
  const RefitItem it = items[blockIdx.x];
  const RefitJob j = jobs[it.job];
  const int D = j.q + 1, D3 = D * D * D;
  const Factors<A> f = stage_factors<A>(j.F, D, sm);
  T* S0 = sm + 4 * D * D;
  T* S1 = S0 + D3;
  const TriLists tl = tri_lists_at(S1 + D3, D);
  const int64_t leaf = it.row / j.dof;
  const int l = (int)(it.row - leaf * j.dof);
  load_row<A>(j.vals + it.row * D3, D3, S0);
  const int64_t base = leaf * j.stride + (int64_t)l * nc_of(D);
  refit_row<A>(f, tl, D, S0, S1,
               CoeffOut{j.coeff + base, j.coeff2 ? j.coeff2 + base : nullptr, j.err});
}

// Raise a kernel's dynamic shared-memory limit to the degree-16 size, once
// per device.
template <class K>
void allow_smem(K kernel, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (!(done.load() & bit)) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)refit_smem(TBSLAS_MAX_DEGREE));
    done.fetch_or(bit);
  }
}

std::atomic<uint64_t> g_smem_refit{0}, g_smem_refit_df{0}, g_smem_refit_t{0},
    g_smem_refit_t_df{0}, g_smem_batch{0}, g_smem_batch_f64{0};

}  // namespace

void launch_refit(const double* vals, const double* F, int q, int64_t rows, int dof,
                  int64_t stride, double* coeff, float2* coeff2, uint32_t* err, bool df_sums,
                  cudaStream_t s) {
  if (rows <= 0) return;
  if (df_sums) {
    allow_smem(k_refit<ArithDF>, g_smem_refit_df);
    k_refit<ArithDF><<<(unsigned)rows, kRefitThreads, refit_smem(q), s>>>(vals, F, q, dof, stride,
                                                                         coeff, coeff2, err);
  } else {
    allow_smem(k_refit<ArithF64>, g_smem_refit);
    k_refit<ArithF64><<<(unsigned)rows, kRefitThreads, refit_smem(q), s>>>(vals, F, q, dof,
                                                                          stride, coeff, coeff2,
                                                                          err);
  }
}

void launch_refit_t(const double* lam, const double* F, int q, int64_t rows, double* mu,
                    bool df_sums, cudaStream_t s) {
  if (rows <= 0) return;
  if (df_sums) {
    allow_smem(k_refit_t<ArithDF>, g_smem_refit_t_df);
    k_refit_t<ArithDF><<<(unsigned)rows, kRefitThreads, refit_smem(q), s>>>(lam, F, q, mu);
  } else {
    allow_smem(k_refit_t<ArithF64>, g_smem_refit_t);
    k_refit_t<ArithF64><<<(unsigned)rows, kRefitThreads, refit_smem(q), s>>>(lam, F, q, mu);
  }
}

void launch_batch_refit(const RefitJob* jobs, const RefitItem* items, int64_t n_items, int max_q,
                        bool df_sums, cudaStream_t s) {
  if (n_items <= 0) return;
  if (df_sums) {
    allow_smem(k_batch_refit<ArithDF>, g_smem_batch);
    k_batch_refit<ArithDF><<<(unsigned)n_items, kRefitThreads, refit_smem(max_q), s>>>(jobs,
                                                                                       items);
  } else {
    allow_smem(k_batch_refit<ArithF64>, g_smem_batch_f64);
    k_batch_refit<ArithF64><<<(unsigned)n_items, kRefitThreads, refit_smem(max_q), s>>>(jobs,
                                                                                        items);
  }
}

// Split FP64 coefficients into their double-float form.
__global__ void k_split(const double* __restrict__ c, float2* __restrict__ c2, int64_t n,
                        uint32_t* err) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const double x = c[i];
    check_df_range(x, err);
    const df v = df_from_double(x);
    c2[i] = make_float2(v.hi, v.lo);
  }
}

void launch_split(const double* c, float2* c2, int64_t n, uint32_t* err, cudaStream_t s) {
  if (n > 0) k_split<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c, c2, n, err);
}

}  // namespace tbg
