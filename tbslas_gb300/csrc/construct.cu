// Analytic input fields on the device and the uniform starting tree of the
// device tree construction (tbslas_tree_construct / tbslas_tree_fit_field,
// the host sequence in capi.cu): the reference's ConstructTree and InitTree
// (src/tree/tree_utils.h:83-178) evaluate an input function at every leaf's
// Chebyshev nodes and fit it; the input functions of its drivers are the
// closed forms of src/utils/fields.h.
#include "internal.h"

namespace tbg {

namespace {

__device__ __forceinline__ void field_at(int kind, int n, const double* __restrict__ p, double x,
                                         double y, double z, double* v) {
  const double tp = 6.283185307179586;  // 2 pi
  switch (kind) {
    case TBSLAS_FIELD_GAUSSIANS: {  // sum_i amp exp(-|x - c|^2 / (2 sigma^2))
      double s = 0.0;
      for (int i = 0; i < n; ++i) {
        const double* g = p + 5 * i;
        const double dx = x - g[0], dy = y - g[1], dz = z - g[2];
        s += g[4] * exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * g[3] * g[3]));
      }
      v[0] = s;
      break;
    }
    case TBSLAS_FIELD_GAUSSIAN_3D: {  // get_gaussian_field_3d (fields.h:275-294)
      const double dx = x - p[0], dy = y - p[1], dz = z - p[2];
      v[0] = p[3] * exp(-((dx * dx) / (2 * p[4] * p[4]) + (dy * dy) / (2 * p[5] * p[5]) +
                          (dz * dz) / (2 * p[6] * p[6])));
      break;
    }
    case TBSLAS_FIELD_EXP_ALPHA: {  // get_exp_alpha_field (fields.h:28-42)
      const double dx = x - p[0], dy = y - p[1], dz = z - p[2];
      v[0] = exp(-pow(sqrt(dx * dx + dy * dy + dz * dz) / p[3], p[4]));
      break;
    }
    case TBSLAS_FIELD_ROTATION:  // get_vorticity_field (fields.h:142-157), omega = p[0]
      v[0] = p[0] * (0.5 - y);
      v[1] = p[0] * (x - 0.5);
      v[2] = 0.0;
      break;
    case TBSLAS_FIELD_TAYLOR_GREEN:
      v[0] = sin(tp * x) * cos(tp * y) * cos(tp * z);
      v[1] = -cos(tp * x) * sin(tp * y) * cos(tp * z);
      v[2] = 0.0;
      break;
    case TBSLAS_FIELD_TAYLOR_GREEN_ABC:  // get_taylor_green_field (fields.h:51-80)
      v[0] = p[0] * cos(p[3] * x) * sin(p[4] * y) * sin(p[5] * z);
      v[1] = p[1] * sin(p[3] * x) * cos(p[4] * y) * sin(p[5] * z);
      v[2] = p[2] * sin(p[3] * x) * sin(p[4] * y) * cos(p[5] * z);
      break;
    case TBSLAS_FIELD_HOPF: {  // get_hopf_field (fields.h:119-139)
      const double dx = x - p[0], dy = y - p[1], dz = z - p[2], r = p[4];
      const double r2 = dx * dx + dy * dy + dz * dz;
      const double c = p[3] / ((r * r + r2) * (r * r + r2));
      v[0] = c * (2 * (-r * dy + dx * dz));
      v[1] = c * (2 * (r * dx + dy * dz));
      v[2] = c * (r * r - dx * dx - dy * dy + dz * dz);
      break;
    }
    case TBSLAS_FIELD_FOURIER: {  // sum_m A_m cos(2 pi k_m . x) + B_m sin(2 pi k_m . x)
      v[0] = v[1] = v[2] = 0.0;
      for (int i = 0; i < n; ++i) {
        const double* m = p + 9 * i;
        double sn, cs;
        sincos(tp * (m[0] * x + m[1] * y + m[2] * z), &sn, &cs);
        v[0] += m[3] * cs + m[6] * sn;
        v[1] += m[4] * cs + m[7] * sn;
        v[2] += m[5] * cs + m[8] * sn;
      }
      break;
    }
    default:
      v[0] = v[1] = v[2] = 0.0;
  }
}

// out[(leaf * dof + l) * Np + p] = field component l at node p of leaf.
__global__ void k_field_values(int kind, int n, const double* __restrict__ prm,
                               const Geom* __restrict__ geom, int64_t L, const Nodes1D nodes,
                               int D, int dof, double* __restrict__ out) {
  const int64_t NP = (int64_t)D * D * D;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= L * NP) return;
  const int64_t leaf = t / NP;
  const int pnode = (int)(t - leaf * NP);
  const Geom g = geom[leaf];
  const double h = leaf_side(g);
  const double x = g.x + h * nodes.x[pnode % D];
  const double y = g.y + h * nodes.x[(pnode / D) % D];
  const double z = g.z + h * nodes.x[pnode / (D * D)];
  double v[3];
  field_at(kind, n, prm, x, y, z, v);
  for (int l = 0; l < dof; ++l) out[(leaf * dof + l) * NP + pnode] = v[l];
}

// The 8^d leaves of the uniform tree of depth d, in Morton order.
__global__ void k_uniform_leaves(int d, uint64_t* __restrict__ keys, Geom* __restrict__ geom) {
  const int64_t L = 1ll << (3 * d);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L) return;
  const uint64_t key = (uint64_t)i << (3 * (kKeyBits - d));
  uint64_t a[3] = {0, 0, 0};
  for (int b = 0; b < d; ++b)
    for (int ax = 0; ax < 3; ++ax) a[ax] |= ((uint64_t)(i >> (3 * b + ax)) & 1ull) << b;
  keys[i] = key;
  geom[i] = Geom{ldexp((double)a[0], -d), ldexp((double)a[1], -d), ldexp((double)a[2], -d),
                 ldexp(2.0, d)};
}

// Midpoints of the in-situ step's first RK2 stage from the node-grid velocity:
// the arithmetic of rk2_backtrace_from_node (X wrapped in place, then one
// fused multiply-add per axis).
__global__ void k_midpoints(const TreeView con, const Nodes1D nodes, int D, double tau,
                            int periodic, const double* __restrict__ vn,
                            double* __restrict__ xmid) {
  const int64_t NP = (int64_t)D * D * D;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= con.L * NP) return;
  const int64_t leaf = t / NP;
  const int p = (int)(t - leaf * NP);
  const Geom g = con.geom[leaf];
  const double h = leaf_side(g);
  double X[3] = {g.x + h * nodes.x[p % D], g.y + h * nodes.x[(p / D) % D],
                 g.z + h * nodes.x[p / (D * D)]};
  const double half_tau = 0.5 * tau;
  for (int k = 0; k < 3; ++k) {
    if (periodic) X[k] = wrap1(X[k]);
    xmid[3 * t + k] = fma(half_tau, vn[3 * t + k], X[k]);
  }
}

}  // namespace

void launch_midpoints(const TreeView& con, const Nodes1D& nodes, int q, double tau, int periodic,
                      const double* vn, double* xmid, cudaStream_t s) {
  const int64_t N = con.L * (int64_t)(q + 1) * (q + 1) * (q + 1);
  if (N > 0)
    k_midpoints<<<(unsigned)((N + 127) / 128), 128, 0, s>>>(con, nodes, q + 1, tau, periodic, vn,
                                                            xmid);
}

void launch_field_values(int kind, int n, const double* prm, const Geom* geom, int64_t L,
                         const Nodes1D& nodes, int q, int dof, double* out, cudaStream_t s) {
  const int64_t N = L * (int64_t)(q + 1) * (q + 1) * (q + 1);
  if (N > 0)
    k_field_values<<<(unsigned)((N + 127) / 128), 128, 0, s>>>(kind, n, prm, geom, L, nodes, q + 1,
                                                              dof, out);
}

void launch_uniform_leaves(int d, uint64_t* keys, Geom* geom, cudaStream_t s) {
  const int64_t L = 1ll << (3 * d);
  k_uniform_leaves<<<(unsigned)((L + 255) / 256), 256, 0, s>>>(d, keys, geom);
}

}  // namespace tbg
