// ew_api.cu -- the C ABI (include/exwave_gb300.h): context set-up (mesh
// validation, flattening of geometry and materials to device arrays), the
// integrator drivers that sequence the fused kernels, and the small
// non-hot kernels (projection of initial fields, L2 errors, vector update).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/exwave_gb300.h"
#include "ew_basis.h"
#include "ew_hostplan.h"
#include "ew_ff.cuh"
#include "ew_internal.h"
#include "ew_launch.h"

namespace ew {

namespace {
KernelTable g_tables[2][EW_MAX_DEGREE + 2];
std::once_flag g_tables_once;

#define EW_REG(d, n) kernel_table_d##d##_##n(g_tables[d - 2][n]);
void init_tables() {
  EW_REG(2, 2) EW_REG(2, 3) EW_REG(2, 4) EW_REG(2, 5) EW_REG(2, 6) EW_REG(2, 7) EW_REG(2, 8)
  EW_REG(2, 9) EW_REG(2, 10) EW_REG(2, 11) EW_REG(2, 12) EW_REG(2, 13)
  EW_REG(3, 2) EW_REG(3, 3) EW_REG(3, 4) EW_REG(3, 5) EW_REG(3, 6) EW_REG(3, 7) EW_REG(3, 8)
  EW_REG(3, 9) EW_REG(3, 10) EW_REG(3, 11) EW_REG(3, 12) EW_REG(3, 13)
}
#undef EW_REG
}  // namespace

const KernelTable& kernel_table(int dim, int np) {
  std::call_once(g_tables_once, init_tables);
  return g_tables[dim - 2][np];
}

namespace {
// per (dim, degree, precision: FP64 / mixed / compensated): cells per block
// and neighbour staging of the line kernel
int g_tuned[2][EW_MAX_DEGREE + 1][3] = {};
int g_tuned_staging[2][EW_MAX_DEGREE + 1][3] = {};
std::mutex g_tuned_mutex;
}  // namespace

int tuned_cells_per_block(int dim, int degree, int precision) {
  if (dim < 2 || dim > 3 || degree < 1 || degree > EW_MAX_DEGREE || precision < 0 || precision > 2)
    return 0;
  std::lock_guard<std::mutex> lk(g_tuned_mutex);
  return g_tuned[dim - 2][degree][precision];
}

int tuned_staging(int dim, int degree, int precision) {
  if (dim < 2 || dim > 3 || degree < 1 || degree > EW_MAX_DEGREE || precision < 0 || precision > 2)
    return 0;
  std::lock_guard<std::mutex> lk(g_tuned_mutex);
  return g_tuned_staging[dim - 2][degree][precision];
}

cudaError_t upload_cart_constants(int dim, int np) {
  GaussRule g = gauss_rule(np);
  std::vector<double> D(np * np), L0(np), L1(np);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) D[i * np + j] = lagrange_deriv(g.x, j, g.x[i]);
  for (int j = 0; j < np; ++j) {
    L0[j] = lagrange(g.x, j, 0.0);
    L1[j] = lagrange(g.x, j, 1.0);
  }
  return kernel_table(dim, np).set_constants(g.w.data(), D.data(), L0.data(), L1.data());
}

namespace {
thread_local std::string g_create_error;

constexpr int kMaxModes = 8;
struct Modes {
  int n;
  double amp[kMaxModes];
  int k[kMaxModes][3];
};

// ---------------------------------------------------------------- kernels
// y += c x
__global__ void axpy_kernel(int64_t n, double c, const double* x, double* y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] += c * x[i];
}

// y = alpha y + (beta x + gamma z); a NULL x or z drops its term, alpha == 0
// does not read y
__global__ void vec_update_kernel(int64_t n, double alpha, double* y, double beta, const double* x,
                                  double gamma, const double* z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double xz = (x ? beta * x[i] : 0.0) + (z ? gamma * z[i] : 0.0);
    y[i] = alpha == 0.0 ? xz : alpha * y[i] + xz;
  }
}

__global__ void rk_update_kernel(int64_t n, double f1, double f2, int is_last, const double* v1,
                                 double* v2, double* v3) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (is_last) {
      v2[i] = v3[i] + f1 * v1[i];
    } else {
      const double up = v1[i];
      const double a = v2[i] + f1 * up;
      v2[i] = a;
      v3[i] = a + f2 * up;
    }
  }
}

__device__ void map_point_dev(int dim, const double* V, const double* xi, double* x) {
  const int nv = 1 << dim;
  for (int i = 0; i < dim; ++i) x[i] = 0.0;
  for (int v = 0; v < nv; ++v) {
    double phi = 1.0;
    for (int e = 0; e < dim; ++e) phi *= ((v >> e) & 1) ? xi[e] : 1.0 - xi[e];
    for (int i = 0; i < dim; ++i) x[i] += V[v * dim + i] * phi;
  }
}

__device__ double jac_det_dev(int dim, const double* V, const double* xi) {
  const int nv = 1 << dim;
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int v = 0; v < nv; ++v)
    for (int j = 0; j < dim; ++j) {
      double dphi = ((v >> j) & 1) ? 1.0 : -1.0;
      for (int e = 0; e < dim; ++e)
        if (e != j) dphi *= ((v >> e) & 1) ? xi[e] : 1.0 - xi[e];
      for (int i = 0; i < dim; ++i) J[i][j] += V[v * dim + i] * dphi;
    }
  if (dim == 2) return J[0][0] * J[1][1] - J[0][1] * J[1][0];
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

__device__ void membrane_dev(int dim, const Modes& ms, const double* x, double t, double* out) {
  const double pi = 3.14159265358979323846;
  for (int f = 0; f <= dim; ++f) out[f] = 0.0;
  for (int m = 0; m < ms.n; ++m) {
    double ksq = 0.0;
    for (int d = 0; d < dim; ++d) ksq += (double)ms.k[m][d] * ms.k[m][d];
    const double w = pi * sqrt(ksq);
    double prod = 1.0;
    for (int d = 0; d < dim; ++d) prod *= sin(ms.k[m][d] * pi * x[d]);
    out[dim] += ms.amp[m] * cos(w * t) * prod;
    for (int c = 0; c < dim; ++c) {
      double v = -ms.amp[m] * (ms.k[m][c] * pi / w) * sin(w * t);
      for (int d = 0; d < dim; ++d)
        v *= (d == c) ? cos(ms.k[m][d] * pi * x[d]) : sin(ms.k[m][d] * pi * x[d]);
      out[c] += v;
    }
  }
}

// physical coordinates of the Gauss points: one thread per (cell, point)
__global__ void qpoints_kernel(const double* verts, int64_t n_cells, int dim, int np,
                               const double* nodes, double* xyz) {
  int N = 1;
  for (int d = 0; d < dim; ++d) N *= np;
  const int64_t total = n_cells * N;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / N;
    int q = (int)(idx - c * N);
    double xi[3] = {0, 0, 0};
    for (int e = 0; e < dim; ++e) {
      xi[e] = nodes[q % np];
      q /= np;
    }
    map_point_dev(dim, verts + c * (1 << dim) * dim, xi, xyz + idx * dim);
  }
}

__global__ void project_membrane_kernel(const double* verts, int64_t n_cells, int dim, int np,
                                        const double* nodes, Modes ms, double t, double* u) {
  int N = 1;
  for (int d = 0; d < dim; ++d) N *= np;
  const int F = dim + 1;
  const int64_t total = n_cells * N;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / N;
    const int q0 = (int)(idx - c * N);
    int q = q0;
    double xi[3] = {0, 0, 0}, x[3] = {0, 0, 0}, ex[4];
    for (int e = 0; e < dim; ++e) {
      xi[e] = nodes[q % np];
      q /= np;
    }
    map_point_dev(dim, verts + c * (1 << dim) * dim, xi, x);
    membrane_dev(dim, ms, x, t, ex);
    for (int f = 0; f < F; ++f) u[c * F * N + f * N + q0] = ex[f];
  }
}

__global__ void project_gaussian_kernel(const double* verts, int64_t n_cells, int dim, int np,
                                        const double* nodes, double x0, double x1, double x2,
                                        double width, double amp, double* u) {
  int N = 1;
  for (int d = 0; d < dim; ++d) N *= np;
  const int F = dim + 1;
  const int64_t total = n_cells * N;
  const double c0[3] = {x0, x1, x2};
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / N;
    const int q0 = (int)(idx - c * N);
    int q = q0;
    double xi[3] = {0, 0, 0}, x[3] = {0, 0, 0};
    for (int e = 0; e < dim; ++e) {
      xi[e] = nodes[q % np];
      q /= np;
    }
    map_point_dev(dim, verts + c * (1 << dim) * dim, xi, x);
    double r2 = 0.0;
    for (int e = 0; e < dim; ++e) r2 += (x[e] - c0[e]) * (x[e] - c0[e]);
    for (int f = 0; f < dim; ++f) u[c * F * N + f * N + q0] = 0.0;
    u[c * F * N + dim * N + q0] = amp * exp(-r2 / (2.0 * width * width));
  }
}

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) s += red[i];
  return s;
}

// L2 norms with QGauss(k+2): values interpolated from the k+1 Gauss points
// (interp[m][np]), exact solution given by `ms` (mode 0) or a second state
// (mode 1: difference a - b).  acc[0..2] += per-block sums.
__global__ void l2_kernel(const double* verts, int64_t n_cells, int dim, int np, int m,
                          const double* interp, const double* qx, const double* qw, const double* a,
                          const double* b, Modes ms, double t, int mode, double* acc) {
  __shared__ double red[32];
  int N = 1, M = 1;
  for (int d = 0; d < dim; ++d) {
    N *= np;
    M *= m;
  }
  const int F = dim + 1;
  const int64_t total = n_cells * M;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / M;
    int p = (int)(idx - c * M);
    int ia[3] = {0, 0, 0};
    double xi[3] = {0, 0, 0}, w = 1.0;
    for (int e = 0; e < dim; ++e) {
      ia[e] = p % m;
      p /= m;
      xi[e] = qx[ia[e]];
      w *= qw[ia[e]];
    }
    double va[4] = {0, 0, 0, 0}, vb[4] = {0, 0, 0, 0};
    for (int q = 0; q < N; ++q) {
      int qq = q;
      double wgt = 1.0;
      for (int e = 0; e < dim; ++e) {
        wgt *= interp[ia[e] * np + qq % np];
        qq /= np;
      }
      for (int f = 0; f < F; ++f) {
        va[f] += wgt * a[c * F * N + f * N + q];
        if (mode == 1) vb[f] += wgt * b[c * F * N + f * N + q];
      }
    }
    const double* V = verts + c * (1 << dim) * dim;
    const double jxw = fabs(jac_det_dev(dim, V, xi)) * w;
    if (mode == 0) {
      double x[3] = {0, 0, 0};
      map_point_dev(dim, V, xi, x);
      membrane_dev(dim, ms, x, t, vb);
    }
    const double dp = va[dim] - vb[dim];
    s0 += dp * dp * jxw;
    for (int d = 0; d < dim; ++d) {
      const double dv = va[d] - vb[d];
      s1 += dv * dv * jxw;
    }
    s2 += vb[dim] * vb[dim] * jxw;
  }
  const double r0 = block_sum(s0, red);
  const double r1 = block_sum(s1, red);
  const double r2 = block_sum(s2, red);
  if (threadIdx.x == 0) {
    atomicAdd(acc, r0);
    atomicAdd(acc + 1, r1);
    atomicAdd(acc + 2, r2);
  }
}

// inverse transpose of the multilinear map's Jacobian (FP64): returns det J,
// JiT[d][e] = d xi_e / d x_d
__device__ double jac_inv_t_dev(int dim, const double* V, const double* xi, double JiT[3][3]) {
  const int nv = 1 << dim;
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int v = 0; v < nv; ++v)
    for (int j = 0; j < dim; ++j) {
      double dphi = ((v >> j) & 1) ? 1.0 : -1.0;
      for (int e = 0; e < dim; ++e)
        if (e != j) dphi *= ((v >> e) & 1) ? xi[e] : 1.0 - xi[e];
      for (int i = 0; i < dim; ++i) J[i][j] += V[v * dim + i] * dphi;
    }
  if (dim == 2) {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    JiT[0][0] = J[1][1] / det;
    JiT[0][1] = -J[1][0] / det;
    JiT[1][0] = -J[0][1] / det;
    JiT[1][1] = J[0][0] / det;
    return det;
  }
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2],
               c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0], c10 = J[0][2] * J[2][1] - J[0][1] * J[2][2],
               c11 = J[0][0] * J[2][2] - J[0][2] * J[2][0], c12 = J[0][1] * J[2][0] - J[0][0] * J[2][1],
               c20 = J[0][1] * J[1][2] - J[0][2] * J[1][1], c21 = J[0][2] * J[1][0] - J[0][0] * J[1][2],
               c22 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  JiT[0][0] = c00 / det; JiT[0][1] = c01 / det; JiT[0][2] = c02 / det;
  JiT[1][0] = c10 / det; JiT[1][1] = c11 / det; JiT[1][2] = c12 / det;
  JiT[2][0] = c20 / det; JiT[2][1] = c21 / det; JiT[2][2] = c22 / det;
  return det;
}

// sum over the block, returned to every thread (red: 33 doubles)
__device__ double block_sum_all(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) s += red[i];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// Post-processed pressure (WaveEquationOperation::compute_post_pressure,
// wave_equation_operations.cc:784-848) and its L2 error against the
// membrane solution (explicit_wave.cc:476-484).  One block per cell, one
// thread per point of QGauss(k+2) (m = k+2 per direction, Mp = m^dim): the
// Q_{k+1} pressure p* held by its values there solves
// (grad phi, grad p*) = (grad phi, -rho du/dt) with the reference's
// unpreconditioned CG (first unknown constrained, relative tolerance 1e-11,
// at most 6 Mp iterations), is shifted to the mean of p and compared with
// the exact pressure by QGauss(k+3).  Basis data in `pb`: interp (m x np),
// qx (m), qw (m), D (m x m, derivative of the Lagrange basis at qx),
// Ie ((m+1) x m, to the QGauss(k+3) points), ex (m+1), ew (m+1).  The block
// is Mp rounded up to whole warps; the padding threads only join the barriers
// and sums.
__global__ void __launch_bounds__(1024) post_pressure_kernel(const double* verts, const void* mat, int mat_fp64, int dim,
                                     int np, const double* pb, const double* u, const double* dudt,
                                     Modes ms, double t, double* acc) {
  extern __shared__ double ps[];
  const int m = np + 1, me = m + 1, F = dim + 1;
  int N = 1, Mp = 1, Me = 1;
  for (int d = 0; d < dim; ++d) {
    N *= np;
    Mp *= m;
    Me *= me;
  }
  const int64_t c = blockIdx.x;
  const int i = threadIdx.x;
  const bool act = i < Mp;
  const double* interp = pb;
  const double* qx = pb + m * np;
  const double* qw = qx + m;
  const double* D = qw + m;
  const double* Ie = D + m * m;
  const double* ex = Ie + me * m;
  const double* ew = ex + me;
  double* jxw = ps;
  double* met = jxw + Mp;        // 6 per point: (0,0) (1,1) (2,2) (0,1) (0,2) (1,2)
  double* x = met + 6 * Mp;
  double* z = x + Mp;
  double* g = z + Mp;            // dim x Mp
  double* red = g + 3 * Mp;      // 33
  const double* V = verts + c * (1 << dim) * dim;
  // materials: 0 FP32, 1 FP64, 2 float pairs
  const double rho_c = mat_fp64 == 1   ? static_cast<const double*>(mat)[4 * c]
                       : mat_fp64 == 2 ? (double)static_cast<const float*>(mat)[8 * c] +
                                             (double)static_cast<const float*>(mat)[8 * c + 1]
                                       : (double)static_cast<const float*>(mat)[4 * c];
  int ii[3] = {0, 0, 0};
  {
    int q = i;
    for (int e = 0; e < dim; ++e) {
      ii[e] = q % m;
      q /= m;
    }
  }
  const int str[3] = {1, m, m * m};
  // geometry, du/dt and p at this thread's point
  double xi[3] = {0, 0, 0}, w = 1.0;
  for (int e = 0; e < dim; ++e) {
    xi[e] = qx[ii[e]];
    w *= qw[ii[e]];
  }
  double JiT[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  const double jw = act ? fabs(jac_inv_t_dev(dim, V, xi, JiT)) * w : 0.0;
  double vt[3] = {0, 0, 0}, pq = 0.0;
  if (act) {
    jxw[i] = jw;
    double mt[3][3];
    for (int e = 0; e < 3; ++e)
      for (int f = 0; f < 3; ++f) {
        double s = 0.0;
        for (int d = 0; d < dim; ++d) s += JiT[d][e] * JiT[d][f];
        mt[e][f] = jw * s;
      }
    met[6 * i + 0] = mt[0][0];
    met[6 * i + 1] = mt[1][1];
    met[6 * i + 2] = mt[2][2];
    met[6 * i + 3] = mt[0][1];
    met[6 * i + 4] = mt[0][2];
    met[6 * i + 5] = mt[1][2];
    for (int q = 0; q < N; ++q) {
      int qq = q;
      double wgt = 1.0;
      for (int e = 0; e < dim; ++e) {
        wgt *= interp[ii[e] * np + qq % np];
        qq /= np;
      }
      for (int d = 0; d < dim; ++d) vt[d] += wgt * dudt[(c * F + d) * N + q];
      pq += wgt * u[(c * F + dim) * N + q];
    }
    // rhs: reference-coordinate flux jxw JiT^T (-rho du/dt), then D^T
    for (int e = 0; e < dim; ++e) {
      double s = 0.0;
      for (int d = 0; d < dim; ++d) s += JiT[d][e] * (-rho_c * vt[d]);
      g[e * Mp + i] = jw * s;
    }
  }
  __syncthreads();
  auto dtrans = [&](int idx) {
    double s = 0.0;
    for (int e = 0; e < dim; ++e)
      for (int a = 0; a < m; ++a) s += D[a * m + ii[e]] * g[e * Mp + idx + (a - ii[e]) * str[e]];
    return s;
  };
  const double rhs_i = (i == 0 || !act) ? 0.0 : dtrans(i);
  const double vol = block_sum_all(jw, red);
  const double pint = block_sum_all(jw * pq, red);
  // SolverCGvect::solve (elementwise_cg.templates.h:64-145)
  const double ABS_TOL = 1e-20, REL_TOL = 1e-11;
  double xi_v = 0.0;
  double ri = rhs_i;
  const double r0 = sqrt(block_sum_all(ri * ri, red));
  if (r0 > 0.0) {
    double pi_v = ri;
    double ry = block_sum_all(ri * pi_v, red);
    for (int it = 1; it <= 6 * Mp; ++it) {
      // v = K p with unknown 0 constrained
      if (act) z[i] = (i == 0) ? 0.0 : pi_v;
      __syncthreads();
      double g0 = 0.0, g1 = 0.0, g2 = 0.0;
      if (act) {
        double gr[3] = {0, 0, 0};
        for (int e = 0; e < dim; ++e)
          for (int a = 0; a < m; ++a) gr[e] += D[ii[e] * m + a] * z[i + (a - ii[e]) * str[e]];
        const double* mt = met + 6 * i;
        g0 = mt[0] * gr[0] + mt[3] * gr[1] + mt[4] * gr[2];
        g1 = mt[3] * gr[0] + mt[1] * gr[1] + mt[5] * gr[2];
        g2 = mt[4] * gr[0] + mt[5] * gr[1] + mt[2] * gr[2];
      }
      __syncthreads();
      if (act) {
        g[i] = g0;
        if (dim > 1) g[Mp + i] = g1;
        if (dim > 2) g[2 * Mp + i] = g2;
      }
      __syncthreads();
      const double vi = !act ? 0.0 : (i == 0) ? pi_v : dtrans(i);
      double pvv = block_sum_all(pi_v * vi, red);
      if (fabs(pvv) < ABS_TOL) pvv = ABS_TOL;
      const double alpha = ry / pvv;
      xi_v += alpha * pi_v;
      ri -= alpha * vi;
      const double rr = block_sum_all(ri * ri, red);
      const double rn = sqrt(rr);
      if (rn < ABS_TOL || rn / r0 < REL_TOL) break;
      const double beta = rr / ry;
      pi_v = ri + beta * pi_v;
      ry = rr;
    }
  }
  // mean of p
  const double sint = block_sum_all(jw * xi_v, red);
  if (act) x[i] = xi_v + (pint - sint) / vol;
  __syncthreads();
  // L2 error with QGauss(k+3)
  double es = 0.0;
  for (int q = i; q < Me; q += blockDim.x) {
    int ie[3] = {0, 0, 0}, tq = q;
    double xe[3] = {0, 0, 0}, we = 1.0;
    for (int e = 0; e < dim; ++e) {
      ie[e] = tq % me;
      tq /= me;
      xe[e] = ex[ie[e]];
      we *= ew[ie[e]];
    }
    double val = 0.0;
    for (int a = 0; a < Mp; ++a) {
      int aa = a;
      double wgt = 1.0;
      for (int e = 0; e < dim; ++e) {
        wgt *= Ie[ie[e] * m + aa % m];
        aa /= m;
      }
      val += wgt * x[a];
    }
    double xp[3] = {0, 0, 0}, exv[4];
    map_point_dev(dim, V, xe, xp);
    membrane_dev(dim, ms, xp, t, exv);
    const double d = val - exv[dim];
    es += d * d * fabs(jac_det_dev(dim, V, xe)) * we;
  }
  const double tot = block_sum_all(es, red);
  if (i == 0) atomicAdd(acc + 3, tot);
}

int grid_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 1 << 20);
}

}  // namespace
}  // namespace ew

// ================================================================ context
// ew_lsrk45_step_host copies the state in this many chunks per direction
constexpr int kHostChunks = 16;

struct ew_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  int dim = 0, degree = 0, np = 0, N = 0, F = 0;
  int64_t n_cells = 0, n_dofs = 0;
  bool mixed = false, cart = false, post = false;
  bool ff = false;  // compensated operator (float-float arithmetic, FP32 data)
  // axis-aligned cells served by the line kernel (it is built for every
  // degree in 2-D and up to degree 7 in 3-D; otherwise the generic kernel)
  bool line = false;
  bool nb_lines = false;  // line kernel: per-thread neighbour lines even where bulk copies are built
  bool spectral = true;  // ADER: spectral evaluation with degree reduction
  int cb_stage = 1, cb_ck = 1;
  const ew::KernelTable* kt = nullptr;
  int32_t* d_nbr = nullptr;
  void* d_geo = nullptr;
  void* d_mat = nullptr;
  double* d_verts = nullptr;
  void* d_basis = nullptr;
  double* d_nodes = nullptr;
  ew::WorkItem* d_work_stage = nullptr;
  int n_work_stage = 0;
  ew::WorkItem* d_work_ck = nullptr;
  int n_work_ck = 0;
  void* d_cellc = nullptr;  // Cartesian kernel per-cell constants
  ew::WorkItem* d_work_cart = nullptr;
  int n_work_cart = 0;
  int cb_cart = 1;
  // line kernel launches over the work items [wr_begin, wr_begin + wr_count)
  // only (wr_count < 0: all)
  int wr_begin = 0, wr_count = -1;
  int grid_stage[ew::N_STAGE_VARIANTS] = {0, 0, 0};
  int grid_ck = 0;
  int* d_err = nullptr;
  double* d_tmp64 = nullptr;
  float* d_x32[2] = {nullptr, nullptr};
  double* d_acc = nullptr;
  double* d_l2 = nullptr;  // interp (m x np), qx (m), qw (m)
  int l2_m = 0;
  // receivers (ew_set_receivers): cell and N interpolation weights each
  int32_t n_rec = 0;
  int32_t* d_rec_cell = nullptr;
  double* d_rec_w = nullptr;
  // ADERADCONFULL: two FP64 vectors for the repeated operator applications
  // (the first also holds du/dt of the post-processing)
  double* d_ad[2] = {nullptr, nullptr};
  double* d_post = nullptr;  // basis data of the post-processing (QGauss(k+2), QGauss(k+3))
  // ew_lsrk45_step_host: the state's two device vectors, the two copy
  // streams and the events that order them (created on first use)
  double* d_hstate[2] = {nullptr, nullptr};
  cudaStream_t s_h2d = nullptr, s_d2h = nullptr;
  cudaEvent_t ev_entry = nullptr, ev_h2d = nullptr, ev_step = nullptr;
  cudaEvent_t ev_d2h[kHostChunks] = {};
  // the host step's compute runs on its own stream: ev_comp marks its end
  // (every other entry point orders the context stream after it), and
  // ev_nfree[k] the point after which the step no longer touches chunk k of
  // the device state d_hstate[0], so that the next call's copy in of that
  // chunk may start
  cudaStream_t s_comp = nullptr;
  cudaEvent_t ev_comp = nullptr;
  cudaEvent_t ev_nfree[kHostChunks] = {};
  bool comp_pending = false, nfree_valid = false;
  cudaEvent_t ev_in[kHostChunks] = {};  // input chunk on the device (and split)
  cudaEvent_t ev_s5[kHostChunks] = {};  // last stage done on the chunk
  // the chunks: with the line kernel, runs of whole work items, and the
  // input chunks that hold their cells' neighbours (lo..hi); else equal
  // runs of DoFs
  std::vector<ew::HostChunk> hchunks;
  // every chunk's neighbours lie in the chunk itself or the two next to it:
  // all five stages can run chunk by chunk as a wavefront
  bool host_wave = false;
  const double* last_host_out = nullptr;  // host output of the previous host step
  bool d2h_pending = false;
  std::string last_error;
  int64_t launches = 0;
};

namespace {

int fail(ew_ctx* c, int code, const std::string& msg) {
  if (c)
    c->last_error = msg;
  else
    ew::g_create_error = msg;
  return code;
}

int cuda_fail(ew_ctx* c, cudaError_t e, const char* what) {
  return fail(c, EW_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
int dev_alloc(ew_ctx* c, T** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(c, EW_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  return EW_OK;
}

int upload(ew_ctx* c, void* dst, const void* src, size_t bytes) {
  cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpy");
  return EW_OK;
}

void free_ctx(ew_ctx* c) {
  if (!c) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  if (c->s_comp) cudaStreamSynchronize(c->s_comp);
  if (c->s_d2h) cudaStreamSynchronize(c->s_d2h);
  if (c->s_h2d) cudaStreamSynchronize(c->s_h2d);
  void* ptrs[] = {c->d_nbr, c->d_geo, c->d_mat, c->d_verts, c->d_basis, c->d_nodes,
                  c->d_work_stage, c->d_work_ck, c->d_work_cart, c->d_cellc, c->d_err, c->d_tmp64, c->d_x32[0],
                  c->d_x32[1], c->d_acc, c->d_l2, c->d_rec_cell, c->d_rec_w, c->d_ad[0], c->d_ad[1], c->d_post,
                  c->d_hstate[0], c->d_hstate[1]};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  cudaEvent_t evs[] = {c->ev_entry, c->ev_h2d, c->ev_step, c->ev_comp};
  for (cudaEvent_t e : evs)
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < kHostChunks; ++k)
    for (cudaEvent_t e : {c->ev_d2h[k], c->ev_in[k], c->ev_s5[k], c->ev_nfree[k]})
      if (e) cudaEventDestroy(e);
  if (c->s_h2d) cudaStreamDestroy(c->s_h2d);
  if (c->s_d2h) cudaStreamDestroy(c->s_d2h);
  if (c->s_comp) cudaStreamDestroy(c->s_comp);
  cudaSetDevice(prev);
  delete c;
}

// Checks of the mesh description (the reference relies on deal.II's
// Triangulation for these invariants).
int validate_mesh_impl(const ew_mesh_desc* m, bool* cartesian) {
  if (!m) return fail(nullptr, EW_ERR_INVALID, "mesh is NULL");
  if (m->dim != 2 && m->dim != 3) return fail(nullptr, EW_ERR_INVALID, "dim must be 2 or 3");
  if (m->degree < 1 || m->degree > EW_MAX_DEGREE)
    return fail(nullptr, EW_ERR_INVALID, "degree must be in 1.." + std::to_string(EW_MAX_DEGREE));
  if (m->n_cells < 1 || m->n_cells > (int64_t)0x7fffffff)
    return fail(nullptr, EW_ERR_INVALID, "n_cells out of range");
  if (!m->vertices || !m->neighbors || !m->speed || !m->density)
    return fail(nullptr, EW_ERR_INVALID, "mesh arrays must not be NULL");
  const int dim = m->dim, nv = 1 << dim, nf = 2 * dim;
  bool cart = true;
  for (int64_t c = 0; c < m->n_cells; ++c) {
    if (!(m->speed[c] > 0.0) || !(m->density[c] > 0.0) || !std::isfinite(m->speed[c]) ||
        !std::isfinite(m->density[c]))
      return fail(nullptr, EW_ERR_INVALID, "speed and density must be positive, cell " +
                                               std::to_string(c));
    const double* V = m->vertices + (size_t)c * nv * dim;
    double scale = 0.0;
    for (int e = 0; e < dim; ++e) scale = std::max(scale, std::fabs(V[(nv - 1) * dim + e] - V[e]));
    if (!(scale > 0.0)) return fail(nullptr, EW_ERR_INVALID, "degenerate cell " + std::to_string(c));
    for (int v = 0; v < nv && cart; ++v)
      for (int e = 0; e < dim; ++e) {
        const double ref = ((v >> e) & 1) ? V[(nv - 1) * dim + e] : V[e];
        if (V[v * dim + e] != ref) cart = false;
      }
    for (int f = 0; f < nf; ++f) {
      const int32_t nb = m->neighbors[c * nf + f];
      if (nb < 0) {
        if (nb < -3)
          return fail(nullptr, EW_ERR_INVALID,
                      "boundary id must be 1, 2 or 3 (cell " + std::to_string(c) + ")");
        continue;
      }
      if (nb >= m->n_cells)
        return fail(nullptr, EW_ERR_INVALID, "neighbor index out of range, cell " + std::to_string(c));
      if (m->neighbors[(int64_t)nb * nf + (f ^ 1)] != (int32_t)c)
        return fail(nullptr, EW_ERR_INVALID,
                    "neighbor relation not symmetric at cell " + std::to_string(c));
      // the shared face must have the same vertices in the same tangential order
      const int e = f / 2, s = f % 2;
      const double* W = m->vertices + (size_t)nb * nv * dim;
      for (int v = 0; v < nv; ++v) {
        if (((v >> e) & 1) != s) continue;
        const int w = v ^ (1 << e);
        for (int d = 0; d < dim; ++d)
          if (std::fabs(V[v * dim + d] - W[w * dim + d]) > 1e-10 * scale)
            return fail(nullptr, EW_ERR_INVALID,
                        "face of cell " + std::to_string(c) +
                            " does not match its neighbor in standard orientation");
      }
    }
  }
  *cartesian = cart;
  return EW_OK;
}

}  // namespace

int ew::validate_mesh(const ew_mesh_desc* m, bool* cartesian, std::string* err) {
  const int rc = validate_mesh_impl(m, cartesian);
  if (rc && err) *err = ew::g_create_error;
  return rc;
}

namespace {

template <typename Real>
std::vector<Real> to_real_vec(const std::vector<double>& v) {
  return std::vector<Real>(v.begin(), v.end());
}

int build_work(ew_ctx* c, int cb, ew::WorkItem** d_work, int* n_work) {
  std::vector<ew::WorkItem> w;
  for (int64_t b = 0; b < c->n_cells; b += cb) {
    ew::WorkItem it;
    it.solve = 0;
    it.cell_begin = (int32_t)b;
    it.n_cells = (int32_t)std::min<int64_t>(cb, c->n_cells - b);
    it.pad = 0;
    w.push_back(it);
  }
  int rc = dev_alloc(c, d_work, w.size());
  if (rc) return rc;
  *n_work = (int)w.size();
  return upload(c, *d_work, w.data(), w.size() * sizeof(ew::WorkItem));
}

int default_cb(int points, int requested) {
  if (requested > 0) return std::max(1, std::min(requested, 512 / points));
  return std::max(1, 512 / points);
}

int set_device(ew_ctx* c) {
  if (!c) return EW_ERR_INVALID;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  return EW_OK;
}

// Entry of every operation on the context stream: after the device and, if
// a host step's compute is still running on its own stream, after it (the
// two share the context's scratch vectors).
int check(ew_ctx* c) {
  int rc = set_device(c);
  if (rc) return rc;
  if (c->comp_pending) {
    const cudaError_t e = cudaStreamWaitEvent(c->stream, c->ev_comp, 0);
    if (e != cudaSuccess) return cuda_fail(c, e, "host step ordering");
    c->comp_pending = false;
  }
  return EW_OK;
}

ew::LaunchArgs base_args(ew_ctx* c, bool ck) {
  ew::LaunchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.single.nbr = c->d_nbr;
  a.single.geo = c->d_geo;
  a.single.mat = c->d_mat;
  a.single.cellc = c->d_cellc;
  a.single.src_cell = -1;
  a.single.n_cells = c->n_cells;
  a.single.bf = 1.0f;
  a.solves = nullptr;
  a.work = ck ? c->d_work_ck : c->d_work_stage;
  a.n_work = ck ? c->n_work_ck : c->n_work_stage;
  a.cells_per_block = ck ? c->cb_ck : c->cb_stage;
  a.basis = c->d_basis;
  a.err = c->d_err;
  return a;
}

void split(double v, float* hi, float* lo) {
  *hi = (float)v;
  *lo = (float)(v - (double)*hi);
}

bool cart_variant_in32(int cv) {
  return cv == ew::CV_MIX_APPLY32 || cv == ew::CV_MIX_MID || cv == ew::CV_MIX_LAST ||
         cv == ew::CV_MIX_UPD || cv == ew::CV_MIX_LAST_FF || cv == ew::CV_MIX_S1_FF;
}
bool cart_variant_apply(int cv) {
  return cv == ew::CV_F64_APPLY || cv == ew::CV_MIX_APPLY64 || cv == ew::CV_MIX_APPLY32 ||
         cv == ew::CV_FF_APPLY64 || cv == ew::CV_FF_APPLYFF;
}

// One operator launch.  `variant` selects the general (curved-cell) kernel,
// `cvar` the Cartesian line kernel; the context uses the one that fits its
// mesh.
int launch_stage(ew_ctx* c, int variant, int cvar, const double* A, const void* X, void* Xout,
                 double* Aout, int mode, double f1, double f2, float bf) {
  ew::LaunchArgs a = base_args(c, false);
  a.single.X = X;
  a.single.A = A;
  a.single.Xout = Xout;
  a.single.Aout = Aout;
  a.single.f1 = f1;
  a.single.f2 = f2;
  a.single.f1f = (float)f1;
  split(f1, &a.single.f1_hi, &a.single.f1_lo);
  split(f1 + f2, &a.single.fb_hi, &a.single.fb_lo);
  a.single.bf = bf;
  a.single.mode = mode;
  cudaError_t e;
  if (c->ff) {
    // compensated contexts: the float-float kernels of the same roles
    switch (cvar) {
      case ew::CV_MIX_APPLY64: cvar = ew::CV_FF_APPLY64; break;
      case ew::CV_MIX_S1: cvar = ew::CV_FF_S1; break;
      case ew::CV_MIX_MID: cvar = ew::CV_FF_MID; break;
      case ew::CV_MIX_LAST: cvar = ew::CV_FF_LAST; break;
      case ew::CV_MIX_UPD: cvar = ew::CV_FF_UPD; break;
      case ew::CV_MIX_APPLY32: cvar = ew::CV_FF_APPLYFF; break;
      case ew::CV_FF_LAST_PAIR: break;
      default:
        return fail(c, EW_ERR_UNSUPPORTED, "this operation is not built for EW_PREC_MIXED_FF");
    }
    variant = variant == ew::STAGE_MIX_IN64 ? ew::STAGE_FF_IN64 : ew::STAGE_FF_INFF;
  }
  if (c->line) {
    // line kernel: stage X unless it is the accumulator itself (first LSRK
    // stage); bulk copies need 16-byte alignment
    const size_t in_sz = cart_variant_in32(cvar) ? 4 : 8;
    const size_t a_sz = cvar == ew::CV_MIX_S1_FF ? 4 : 8;  // lo array of a float-pair state
    const bool sa = !cart_variant_apply(cvar);
    const int sx = (sa && static_cast<const void*>(A) == X && in_sz == 8) ? 0 : 1;
    const size_t cell_elems = (size_t)c->F * c->N;
    const bool tma = (cell_elems * in_sz) % 16 == 0 && (cell_elems * a_sz) % 16 == 0 &&
                     (reinterpret_cast<uintptr_t>(X) % 16) == 0 &&
                     (!sa || (reinterpret_cast<uintptr_t>(A) % 16) == 0);
    // the whole work list, or the range set for a chunked launch
    a.work = c->d_work_cart + (c->wr_count >= 0 ? c->wr_begin : 0);
    a.n_work = c->wr_count >= 0 ? c->wr_count : c->n_work_cart;
    a.cells_per_block = c->cb_cart;
    const ew::CartEntry& k = c->kt->cart[cvar];
    const int occ = std::max(1, k.occupancy(c->cb_cart, sx));
    const int grid = std::max(1, std::min(a.n_work, occ * c->num_sms));
    e = k.launch(a, sx, tma ? 1 : 0, c->nb_lines ? 1 : 0, grid, c->stream);
  } else {
    const ew::KernelEntry& k = c->kt->stage[variant][c->cart ? 1 : 0];
    if (!k.launch) return fail(c, EW_ERR_UNSUPPORTED, "no stage kernel built for this mesh and precision");
    e = k.launch(a, c->grid_stage[variant], c->stream);
  }
  ++c->launches;
  if (e != cudaSuccess) return cuda_fail(c, e, "stage kernel launch");
  return EW_OK;
}

// The CK kernel of the context: precision, cell kind, post-processing and
// spectral evaluation (below degree 4 both evaluations are the same kernel).
const ew::KernelEntry& ck_entry(const ew_ctx* c) {
  const int p = c->ff ? 2 : (c->mixed ? 1 : 0), ca = c->cart ? 1 : 0, po = c->post ? 1 : 0;
  return (c->spectral || c->np < 5) ? c->kt->ck[p][ca][po] : c->kt->ck_full[p][ca][po];
}

int launch_ck(ew_ctx* c, double dt, const double* src, void* T) {
  ew::LaunchArgs a = base_args(c, true);
  a.single.X = src;
  a.single.Xout = T;
  a.dt = dt;
  // Taylor coefficients (integrate_taylor_cauchykovalewski_step,
  // wave_equation_operations.cc:1079-1082): fac_s = -1/2 prod_{j=2}^{s+2}
  // (-1/(j+1)), times dt^(s+3)
  a.ck_dt_d = dt;
  a.ck_half_dt2_d = 0.5 * dt * dt;
  a.ck_dt = (float)dt;
  a.ck_half_dt2 = (float)(0.5 * dt * dt);
  double fac = -0.5, dtp = dt * dt * dt;
  for (int s = 0; s < 12; ++s) {
    fac /= -(s + 3.0);
    a.ck_fac_d[s] = fac * dtp;
    a.ck_fac[s] = (float)(fac * dtp);
    dtp *= dt;
  }
  const ew::KernelEntry& k = ck_entry(c);
  if (!k.launch)
    return fail(c, EW_ERR_UNSUPPORTED,
                "ADER: the Cauchy-Kovalevskaya kernel is built for 3-D degrees up to 7 (all degrees in 2-D)");
  cudaError_t e = k.launch(a, c->grid_ck, c->stream);
  ++c->launches;
  if (e != cudaSuccess) return cuda_fail(c, e, "ck kernel launch");
  return EW_OK;
}

}  // namespace

// ================================================================ C ABI
// ---- receivers (helpers) ---------------------------------------------------------------
namespace {
// Multilinear map of a cell (2^dim vertices, lexicographic) and its Jacobian.
void cell_map(int dim, const double* V, const double* xi, double* x, double* J) {
  const int nv = 1 << dim;
  for (int i = 0; i < dim; ++i) {
    x[i] = 0.0;
    for (int j = 0; j < dim; ++j) J[i * dim + j] = 0.0;
  }
  for (int v = 0; v < nv; ++v) {
    double phi = 1.0;
    for (int d = 0; d < dim; ++d) phi *= ((v >> d) & 1) ? xi[d] : 1.0 - xi[d];
    for (int i = 0; i < dim; ++i) x[i] += V[v * dim + i] * phi;
    for (int j = 0; j < dim; ++j) {
      double dp = ((v >> j) & 1) ? 1.0 : -1.0;
      for (int d = 0; d < dim; ++d)
        if (d != j) dp *= ((v >> d) & 1) ? xi[d] : 1.0 - xi[d];
      for (int i = 0; i < dim; ++i) J[i * dim + j] += V[v * dim + i] * dp;
    }
  }
}

// Reference coordinates of point p in a cell by Newton's method on the
// multilinear map; true if p lies in the cell (with a small tolerance).
bool invert_map(int dim, const double* V, const double* p, double* xi) {
  for (int d = 0; d < dim; ++d) xi[d] = 0.5;
  double x[3], J[9];
  for (int it = 0; it < 40; ++it) {
    cell_map(dim, V, xi, x, J);
    double r[3], dx[3] = {0, 0, 0};
    for (int i = 0; i < dim; ++i) r[i] = x[i] - p[i];
    if (dim == 2) {
      const double det = J[0] * J[3] - J[1] * J[2];
      if (det == 0.0) return false;
      dx[0] = (J[3] * r[0] - J[1] * r[1]) / det;
      dx[1] = (-J[2] * r[0] + J[0] * r[1]) / det;
    } else {
      const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8],
                   c02 = J[3] * J[7] - J[4] * J[6];
      const double det = J[0] * c00 + J[1] * c01 + J[2] * c02;
      if (det == 0.0) return false;
      // inverse = adj(J) / det, adj = cofactor matrix transposed
      const double c10 = J[2] * J[7] - J[1] * J[8], c11 = J[0] * J[8] - J[2] * J[6],
                   c12 = J[1] * J[6] - J[0] * J[7];
      const double c20 = J[1] * J[5] - J[2] * J[4], c21 = J[2] * J[3] - J[0] * J[5],
                   c22 = J[0] * J[4] - J[1] * J[3];
      dx[0] = (c00 * r[0] + c10 * r[1] + c20 * r[2]) / det;
      dx[1] = (c01 * r[0] + c11 * r[1] + c21 * r[2]) / det;
      dx[2] = (c02 * r[0] + c12 * r[1] + c22 * r[2]) / det;
    }
    double step = 0.0;
    for (int d = 0; d < dim; ++d) {
      xi[d] -= dx[d];
      step = std::max(step, std::fabs(dx[d]));
    }
    if (step < 1e-14) break;
  }
  for (int d = 0; d < dim; ++d)
    if (!(xi[d] >= -1e-10 && xi[d] <= 1.0 + 1e-10)) return false;
  return true;
}

// One warp per receiver: every field of the state at the receiver.
__global__ void receivers_kernel(const double* state, int n, int F, int N, const int32_t* cell,
                                 const double* w, double* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* wr = w + (size_t)warp * N;
  for (int fld = 0; fld < F; ++fld) {
    const double* s = state + ((size_t)cell[warp] * F + fld) * N;
    double acc = 0.0;
    for (int q = lane; q < N; q += 32) acc += wr[q] * s[q];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) out[(size_t)warp * F + fld] = acc;
  }
}
}  // namespace

extern "C" {

const char* ew_last_error(const ew_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : ew::g_create_error.c_str();
}

int ew_create(const ew_mesh_desc* mesh, const ew_options* options, ew_ctx** out) {
  if (!out) return fail(nullptr, EW_ERR_INVALID, "ctx output pointer is NULL");
  *out = nullptr;
  bool cart = false;
  int rc = validate_mesh_impl(mesh, &cart);
  if (rc) return rc;
  ew_options opt;
  std::memset(&opt, 0, sizeof(opt));
  opt.spectral_evaluation = 1;
  if (options) opt = *options;
  if (opt.precision != EW_PREC_FP64 && opt.precision != EW_PREC_MIXED &&
      opt.precision != EW_PREC_MIXED_FF)
    return fail(nullptr, EW_ERR_INVALID,
                "precision must be EW_PREC_FP64, EW_PREC_MIXED or EW_PREC_MIXED_FF");
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0)
    return fail(nullptr, EW_ERR_CUDA, "no CUDA device available");
  if (opt.device < 0 || opt.device >= ndev) return fail(nullptr, EW_ERR_INVALID, "bad device");

  ew_ctx* c = new ew_ctx;
  c->device = opt.device;
  ce = cudaSetDevice(c->device);
  if (ce != cudaSuccess) {
    delete c;
    return fail(nullptr, EW_ERR_CUDA, "cudaSetDevice failed");
  }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  c->dim = mesh->dim;
  c->degree = mesh->degree;
  c->np = mesh->degree + 1;
  c->F = c->dim + 1;
  c->N = 1;
  for (int d = 0; d < c->dim; ++d) c->N *= c->np;
  c->n_cells = mesh->n_cells;
  c->n_dofs = c->n_cells * c->F * c->N;
  c->mixed = opt.precision != EW_PREC_FP64;
  c->ff = opt.precision == EW_PREC_MIXED_FF;
  c->cart = cart;
  c->post = opt.use_ader_post != 0;
  c->spectral = opt.spectral_evaluation != 0;
  c->kt = &ew::kernel_table(c->dim, c->np);
  c->line = cart && c->kt->cart[ew::CV_F64_MID].launch != nullptr;
  const int dim = c->dim, nv = 1 << dim;

  auto bail = [&](int code) {
    ew::g_create_error = c->last_error;
    free_ctx(c);
    return code;
  };

  // geometry: Cartesian cells keep their extents, others the monomial
  // coefficients of their multilinear map (inclusion-exclusion over the
  // vertices, in FP64: C_S = sum_{T subset S} (-1)^{|S|-|T|} V_T)
  const int geo_per_cell = cart ? dim : nv * dim;
  std::vector<double> geo((size_t)c->n_cells * geo_per_cell);
  for (int64_t i = 0; i < c->n_cells; ++i) {
    const double* V = mesh->vertices + (size_t)i * nv * dim;
    if (cart) {
      for (int e = 0; e < dim; ++e) geo[i * dim + e] = V[(nv - 1) * dim + e] - V[e];
    } else {
      double* C = geo.data() + (size_t)i * nv * dim;
      std::copy(V, V + nv * dim, C);
      for (int d = 0; d < dim; ++d)
        for (int S = 0; S < nv; ++S)
          if ((S >> d) & 1)
            for (int e = 0; e < dim; ++e) C[S * dim + e] -= C[(S ^ (1 << d)) * dim + e];
    }
  }
  // per cell: rho, c, tau = 1/(c rho), 1/rho
  std::vector<double> mat((size_t)c->n_cells * 4);
  for (int64_t i = 0; i < c->n_cells; ++i) {
    mat[4 * i] = mesh->density[i];
    mat[4 * i + 1] = mesh->speed[i];
    mat[4 * i + 2] = 1.0 / (mesh->speed[i] * mesh->density[i]);
    mat[4 * i + 3] = 1.0 / mesh->density[i];
  }
  std::vector<double> basis = ew::basis_table(c->np);
  // Cartesian kernel constants per cell: 1/rho, rho c^2, tau, 1/tau,
  // 1/h_e (3 slots), per face (tau of the neighbour, 1/(tau + tau_nb))
  std::vector<double> cellc;
  if (cart) {
    const int K = 19;
    cellc.assign((size_t)c->n_cells * K, 0.0);
    for (int64_t i = 0; i < c->n_cells; ++i) {
      double* k = &cellc[(size_t)i * K];
      const double rho = mesh->density[i], sp = mesh->speed[i];
      const double tau = 1.0 / (sp * rho);
      k[0] = 1.0 / rho;
      k[1] = rho * sp * sp;
      k[2] = tau;
      k[3] = sp * rho;
      for (int e = 0; e < dim; ++e) k[4 + e] = 1.0 / geo[i * dim + e];
      for (int f = 0; f < 2 * dim; ++f) {
        const int32_t nb = mesh->neighbors[i * 2 * dim + f];
        if (nb < 0) continue;
        const double tm = 1.0 / (mesh->speed[nb] * mesh->density[nb]);
        k[7 + 2 * f] = tm;
        k[8 + 2 * f] = 1.0 / (tau + tm);
      }
    }
  }
  // geometry, materials and basis in the compute type: FP64, FP32 or float pairs
  const size_t rsz = c->mixed && !c->ff ? sizeof(float) : sizeof(double);
  if ((rc = dev_alloc(c, reinterpret_cast<char**>(&c->d_geo), geo.size() * rsz)) ||
      (rc = dev_alloc(c, reinterpret_cast<char**>(&c->d_mat), mat.size() * rsz)) ||
      (rc = dev_alloc(c, reinterpret_cast<char**>(&c->d_basis), basis.size() * rsz)) ||
      (rc = dev_alloc(c, &c->d_nbr, (size_t)c->n_cells * 2 * dim)) ||
      (rc = dev_alloc(c, &c->d_verts, (size_t)c->n_cells * nv * dim)) ||
      (rc = dev_alloc(c, &c->d_nodes, (size_t)c->np)) || (rc = dev_alloc(c, &c->d_err, 4)) ||
      (rc = dev_alloc(c, &c->d_acc, 4)))
    return bail(rc);
  if (c->ff) {
    auto pairs = [](const std::vector<double>& v) {
      std::vector<float> r(v.size() * 2);
      for (size_t i = 0; i < v.size(); ++i) {
        const ew::FF f = ew::FF::from_double(v[i]);
        r[2 * i] = f.hi;
        r[2 * i + 1] = f.lo;
      }
      return r;
    };
    auto g = pairs(geo), m = pairs(mat), b = pairs(basis);
    if ((rc = upload(c, c->d_geo, g.data(), g.size() * 4)) ||
        (rc = upload(c, c->d_mat, m.data(), m.size() * 4)) ||
        (rc = upload(c, c->d_basis, b.data(), b.size() * 4)))
      return bail(rc);
  } else if (c->mixed) {
    auto g = to_real_vec<float>(geo), m = to_real_vec<float>(mat), b = to_real_vec<float>(basis);
    if ((rc = upload(c, c->d_geo, g.data(), g.size() * 4)) ||
        (rc = upload(c, c->d_mat, m.data(), m.size() * 4)) ||
        (rc = upload(c, c->d_basis, b.data(), b.size() * 4)))
      return bail(rc);
  } else {
    if ((rc = upload(c, c->d_geo, geo.data(), geo.size() * 8)) ||
        (rc = upload(c, c->d_mat, mat.data(), mat.size() * 8)) ||
        (rc = upload(c, c->d_basis, basis.data(), basis.size() * 8)))
      return bail(rc);
  }
  if (cart) {
    if ((rc = dev_alloc(c, reinterpret_cast<char**>(&c->d_cellc), cellc.size() * (c->ff ? 8 : rsz))))
      return bail(rc);
    if (c->ff) {
      // each constant as a float pair (hi, lo)
      std::vector<float> f(cellc.size() * 2);
      for (size_t i = 0; i < cellc.size(); ++i) {
        const ew::FF v = ew::FF::from_double(cellc[i]);
        f[2 * i] = v.hi;
        f[2 * i + 1] = v.lo;
      }
      rc = upload(c, c->d_cellc, f.data(), f.size() * 4);
    } else if (c->mixed) {
      auto f = to_real_vec<float>(cellc);
      rc = upload(c, c->d_cellc, f.data(), f.size() * 4);
    } else {
      rc = upload(c, c->d_cellc, cellc.data(), cellc.size() * 8);
    }
    if (rc) return bail(rc);
  }
  if ((rc = upload(c, c->d_nbr, mesh->neighbors, (size_t)c->n_cells * 2 * dim * 4)) ||
      (rc = upload(c, c->d_verts, mesh->vertices, (size_t)c->n_cells * nv * dim * 8)))
    return bail(rc);
  {
    ew::GaussRule g = ew::gauss_rule(c->np);
    if ((rc = upload(c, c->d_nodes, g.x.data(), c->np * 8))) return bail(rc);
    // QGauss(k+2) interpolation data for the L2 errors
    const int m = c->np + 1;
    ew::GaussRule ge = ew::gauss_rule(m);
    std::vector<double> l2(m * c->np + 2 * m);
    for (int a = 0; a < m; ++a)
      for (int i = 0; i < c->np; ++i) l2[a * c->np + i] = ew::lagrange(g.x, i, ge.x[a]);
    std::copy(ge.x.begin(), ge.x.end(), l2.begin() + m * c->np);
    std::copy(ge.w.begin(), ge.w.end(), l2.begin() + m * c->np + m);
    c->l2_m = m;
    if ((rc = dev_alloc(c, &c->d_l2, l2.size())) || (rc = upload(c, c->d_l2, l2.data(), l2.size() * 8)))
      return bail(rc);
  }
  if (cudaMemset(c->d_err, 0, 4 * sizeof(int)) != cudaSuccess)
    return bail(fail(c, EW_ERR_CUDA, "cudaMemset"));

  // even-odd 1D constants of the Cartesian kernel, for this device
  ce = ew::upload_cart_constants(c->dim, c->np);
  if (ce != cudaSuccess) return bail(cuda_fail(c, ce, "constant upload"));
  // work lists and persistent grid sizes
  c->cb_stage = default_cb(c->N, opt.cells_per_block);
  // mixed CK kernel: 80 registers a thread, two blocks per SM need 384 threads or fewer
  c->cb_ck = c->mixed && !c->ff ? std::max(1, std::min(c->cb_stage, 384 / c->N)) : c->cb_stage;
  const ew::KernelEntry& ckk = ck_entry(c);
  while (ckk.smem && c->cb_ck > 1 && ckk.smem(c->cb_ck) > 200 * 1024) --c->cb_ck;
  if (c->line) {
    const int lines = c->kt->lines;
    const int tuned = ew::tuned_cells_per_block(c->dim, c->degree, opt.precision);
    c->cb_cart = opt.cells_per_block > 0 ? opt.cells_per_block
                                         : (tuned > 0 ? tuned : std::max(1, 256 / lines));
    c->cb_cart = std::max(1, std::min(c->cb_cart, std::max(1, 512 / lines)));
    const int v = c->ff ? ew::CV_FF_MID : (c->mixed ? ew::CV_MIX_MID : ew::CV_F64_MID);
    while (c->cb_cart > 1 && c->kt->cart[v].smem(c->cb_cart, 1) > 110 * 1024) --c->cb_cart;
    if (opt.nb_staging < 0 || opt.nb_staging > 2)
      return bail(fail(c, EW_ERR_INVALID, "nb_staging must be 0, 1 or 2"));
    const int staging = opt.nb_staging > 0 ? opt.nb_staging
                                           : ew::tuned_staging(c->dim, c->degree, opt.precision);
    c->nb_lines = staging == 1;
  }
  if ((rc = build_work(c, c->cb_stage, &c->d_work_stage, &c->n_work_stage)) ||
      (rc = build_work(c, c->cb_ck, &c->d_work_ck, &c->n_work_ck)) ||
      (c->line && (rc = build_work(c, c->cb_cart, &c->d_work_cart, &c->n_work_cart))))
    return bail(rc);
  for (int v = 0; v < ew::N_STAGE_VARIANTS; ++v) {
    if (!c->kt->stage[v][cart].occupancy) continue;  // compensated variants: curved cells only
    const int occ = c->kt->stage[v][cart].occupancy(c->cb_stage);
    c->grid_stage[v] = std::max(1, std::min(c->n_work_stage, std::max(occ, 1) * c->num_sms));
  }
  if (ckk.occupancy) {
    const int occ = ckk.occupancy(c->cb_ck);
    c->grid_ck = std::max(1, std::min(c->n_work_ck, std::max(occ, 1) * c->num_sms));
  }
  // integrator scratch: FP64 third register (also the ADER Taylor state);
  // mixed: two FP32 stage inputs (the first also holds the ADER Taylor state);
  // compensated: two stage inputs of float pairs
  if (c->mixed) {
    const size_t per = c->ff ? 2 : 1;
    if ((rc = dev_alloc(c, &c->d_x32[0], (size_t)c->n_dofs * per)) ||
        (rc = dev_alloc(c, &c->d_x32[1], (size_t)c->n_dofs * per)))
      return bail(rc);
  } else {
    if ((rc = dev_alloc(c, &c->d_tmp64, (size_t)c->n_dofs))) return bail(rc);
  }
  ce = cudaDeviceSynchronize();
  if (ce != cudaSuccess) return bail(cuda_fail(c, ce, "set-up"));
  *out = c;
  return EW_OK;
}

void ew_destroy(ew_ctx* ctx) { free_ctx(ctx); }

int ew_set_stream(ew_ctx* ctx, void* stream) {
  if (!ctx) return EW_ERR_INVALID;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return EW_OK;
}

int64_t ew_n_dofs(const ew_ctx* ctx) { return ctx ? ctx->n_dofs : -1; }
int64_t ew_n_cells(const ew_ctx* ctx) { return ctx ? ctx->n_cells : -1; }
int64_t ew_kernel_launches(const ew_ctx* ctx) { return ctx ? ctx->launches : -1; }

int ew_apply(ew_ctx* ctx, const double* src, double* dst) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!src || !dst || src == dst) return fail(ctx, EW_ERR_INVALID, "ew_apply: src/dst invalid");
  const int var = ctx->mixed ? ew::STAGE_MIX_IN64 : ew::STAGE_F64;
  const int cv = ctx->mixed ? ew::CV_MIX_APPLY64 : ew::CV_F64_APPLY;
  return launch_stage(ctx, var, cv, nullptr, src, nullptr, dst, ew::MODE_APPLY, 0.0, 0.0, 1.0f);
}

int ew_rk_update(ew_ctx* ctx, double f1, double f2, int32_t is_last, const double* v1, double* v2,
                 double* v3) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!v1 || !v2 || !v3) return fail(ctx, EW_ERR_INVALID, "ew_rk_update: NULL vector");
  ew::rk_update_kernel<<<ew::grid_for(ctx->n_dofs), 256, 0, ctx->stream>>>(ctx->n_dofs, f1, f2,
                                                                          is_last, v1, v2, v3);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "rk_update launch");
}

namespace {
// The five fused stages of one LowStorageRK45Reg2 step
// (time_integrators.cc:235-283) with the integrator's scratch given by the
// caller: T, the FP64 third register (FP64 path), or X0 / X1, the two stage
// inputs used ping-pong (mixed and compensated paths: FP32 values or float
// pairs).  Shared by ew_lsrk45_step (scratch owned by the context) and
// ew_lsrk45_step_static (scratch in the static device array).
// One stage of the LSRK45 schedule: the arguments of its launch.
struct StageCall {
  int variant, cvar;
  const double* A;
  const void* X;
  void* Xout;
  double* Aout;
  int mode;
  double f1, f2;
};

// The five stages of one LowStorageRK45Reg2 step (time_integrators.cc:235-283)
// on the registers vec_n (the state in; then a register), vec_np (the new
// state), T (FP64 scratch) and X0, X1 (stage inputs of the reduced-precision
// paths).  *split: the compensated Cartesian path first splits the FP64
// state in vec_n in place into float pairs, and its first stage runs as the
// middle-stage kernel on them, like the first stage of a later step in a
// multi-step call (the same exact splits the FP64-input kernel forms on
// load, at 0.6 of its cost).
void lsrk45_plan(const ew_ctx* ctx, double dt, double* vec_n, double* vec_np, double* T, float* X0,
                 float* X1, StageCall st[5], bool* split) {
  using namespace ew;
  const double f1[5] = {kA21 * dt, kA32 * dt, kA43 * dt, kA54 * dt, kB5 * dt};
  const double f2[5] = {(kB1 - kA21) * dt, (kB2 - kA32) * dt, (kB3 - kA43) * dt, (kB4 - kA54) * dt,
                        0.0};
  *split = false;
  if (!ctx->mixed) {
    // Three FP64 registers N = vec_n, P = vec_np, T = scratch.  The stage
    // input is read by neighbouring cells, so the new accumulator goes to
    // the register not read in this stage; the next stage input overwrites
    // the old accumulator in place (cell-local).
    double* N = vec_n;
    double* P = vec_np;
    const double* X[5] = {N, T, P, N, T};
    const double* A[5] = {N, P, N, T, P};
    double* Xo[5] = {T, P, N, T, nullptr};
    double* Ao[5] = {P, N, T, P, P};
    for (int s = 0; s < 5; ++s)
      st[s] = StageCall{STAGE_F64, s < 4 ? CV_F64_MID : CV_F64_LAST, A[s], X[s], Xo[s], Ao[s],
                        s < 4 ? MODE_RK_MID : MODE_RK_LAST, f1[s], f2[s]};
    return;
  }
  // mixed: accumulator in vec_np (in place; on Cartesian meshes a float-float
  // pair between the stages, FP64 at the end), FP32 stage inputs ping-pong
  if (ctx->ff && ctx->line) {
    *split = true;
    st[0] = StageCall{STAGE_MIX_IN32, CV_MIX_MID, vec_n, vec_n, X0, vec_np, MODE_RK_MID, f1[0], f2[0]};
  } else {
    st[0] = StageCall{STAGE_MIX_IN64, CV_MIX_S1, vec_n, vec_n, X0, vec_np, MODE_RK_MID, f1[0], f2[0]};
  }
  const float* xin[4] = {X0, X1, X0, X1};
  float* xout[4] = {X1, X0, X1, nullptr};
  for (int s = 1; s < 5; ++s)
    st[s] = StageCall{STAGE_MIX_IN32, s < 4 ? CV_MIX_MID : CV_MIX_LAST, vec_np, xin[s - 1], xout[s - 1],
                      vec_np, s < 4 ? MODE_RK_MID : MODE_RK_LAST, f1[s], f2[s]};
}

int run_stage(ew_ctx* ctx, const StageCall& s) {
  return launch_stage(ctx, s.variant, s.cvar, s.A, s.X, s.Xout, s.Aout, s.mode, s.f1, s.f2, 1.0f);
}

int split_state(ew_ctx* ctx, double* v, int64_t n, cudaStream_t stream) {
  const cudaError_t e = ew::launch_split_pairs(v, n, v, stream);
  ++ctx->launches;
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "split to float pairs");
}

int lsrk45_stages(ew_ctx* ctx, double dt, double* vec_n, double* vec_np, double* T, float* X0,
                  float* X1) {
  StageCall st[5];
  bool split = false;
  lsrk45_plan(ctx, dt, vec_n, vec_np, T, X0, X1, st, &split);
  int rc;
  if (split && (rc = split_state(ctx, vec_n, ctx->n_dofs, ctx->stream))) return rc;
  for (int s = 0; s < 5; ++s)
    if ((rc = run_stage(ctx, st[s]))) return rc;
  return EW_OK;
}
}  // namespace

int ew_lsrk45_step(ew_ctx* ctx, double dt, double* vec_n, double* vec_np) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!vec_n || !vec_np || vec_n == vec_np)
    return fail(ctx, EW_ERR_INVALID, "ew_lsrk45_step: vec_n and vec_np must be distinct");
  return lsrk45_stages(ctx, dt, vec_n, vec_np, ctx->d_tmp64, ctx->d_x32[0], ctx->d_x32[1]);
}

namespace {
int host_chunk_plan(ew_ctx* c) {
  if (!c->hchunks.empty()) return EW_OK;
  const int64_t cellsz = (int64_t)c->F * c->N;
  if (c->line) {
    const int nf = 2 * c->dim;
    std::vector<int32_t> nbr((size_t)c->n_cells * nf);
    const cudaError_t e =
        cudaMemcpy(nbr.data(), c->d_nbr, nbr.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "neighbour table readback");
    c->host_wave = ew::host_chunk_plan_items(c->n_work_cart, c->cb_cart, c->n_cells, cellsz, nf, nbr.data(),
                                             kHostChunks, &c->hchunks);
  } else {
    const int64_t n = c->n_dofs, chunk = (n + kHostChunks - 1) / kHostChunks;
    for (int k = 0; k < kHostChunks && k * chunk < n; ++k) {
      ew::HostChunk h;
      h.dof_begin = k * chunk;
      h.n_dofs = std::min(chunk, n - k * chunk);
      c->hchunks.push_back(h);
    }
  }
  return EW_OK;
}

// line kernel launches of a scope over one work-item range
struct WorkRange {
  ew_ctx* c;
  WorkRange(ew_ctx* ctx, int begin, int count) : c(ctx) {
    c->wr_begin = begin;
    c->wr_count = count;
  }
  ~WorkRange() {
    c->wr_begin = 0;
    c->wr_count = -1;
  }
};
}  // namespace

int ew_lsrk45_step_host(ew_ctx* ctx, double dt, const double* h_vec_n, double* h_vec_np) {
  // the previous host step's compute is not waited for here: only what it
  // touches is (below)
  int rc = set_device(ctx);
  if (rc) return rc;
  if (!h_vec_n || !h_vec_np) return fail(ctx, EW_ERR_INVALID, "ew_lsrk45_step_host: NULL host vector");
  cudaError_t e = cudaSuccess;
  if (!ctx->d_hstate[0]) {
    if ((rc = dev_alloc(ctx, &ctx->d_hstate[0], (size_t)ctx->n_dofs)) ||
        (rc = dev_alloc(ctx, &ctx->d_hstate[1], (size_t)ctx->n_dofs)))
      return rc;
    const unsigned fl = cudaEventDisableTiming;
    if ((e = cudaStreamCreateWithFlags(&ctx->s_h2d, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->s_d2h, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->s_comp, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->ev_comp, fl)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->ev_entry, fl)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->ev_h2d, fl)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->ev_step, fl)) != cudaSuccess)
      return cuda_fail(ctx, e, "host step streams");
    for (int k = 0; k < kHostChunks; ++k)
      if ((e = cudaEventCreateWithFlags(&ctx->ev_d2h[k], fl)) != cudaSuccess ||
          (e = cudaEventCreateWithFlags(&ctx->ev_in[k], fl)) != cudaSuccess ||
          (e = cudaEventCreateWithFlags(&ctx->ev_s5[k], fl)) != cudaSuccess ||
          (e = cudaEventCreateWithFlags(&ctx->ev_nfree[k], fl)) != cudaSuccess)
        return cuda_fail(ctx, e, "host step events");
  }
  if ((rc = host_chunk_plan(ctx))) return rc;
  const int K = (int)ctx->hchunks.size();
  double* d_n = ctx->d_hstate[0];
  double* d_np = ctx->d_hstate[1];
  StageCall st[5];
  bool split = false;
  lsrk45_plan(ctx, dt, d_n, d_np, ctx->d_tmp64, ctx->d_x32[0], ctx->d_x32[1], st, &split);
  // With the line kernel the stages run chunk by chunk: each chunk of the
  // first stage starts once the input chunks its cells' neighbours lie in
  // have arrived (and are split), and each chunk's copy to the host starts
  // once the last stage has finished that chunk.  The middle stages run as
  // a wavefront over the chunks where every chunk's neighbours lie in the
  // chunks next to it (host_wave), else whole.  The first stage is always
  // the first launch to touch a chunk, after that chunk's input (and so
  // after the previous call's copy out of it, which reads d_np).
  const bool staged = ctx->line;
  // the input chunks that the previous call's output copies are still writing
  const bool chained = ctx->d2h_pending && h_vec_n == ctx->last_host_out;
  auto ordering = [&](cudaError_t err) { return cuda_fail(ctx, err, "host step ordering"); };
  // host -> device, after the work already on the context stream (the
  // caller's, and other operations of the context) and, chunk by chunk,
  // after the previous host step has released that chunk of d_n and copied
  // the same chunk to the host; any other input may still overlap the
  // previous output: after all of it.  The compute, on its own stream, also
  // follows the context stream's work.
  if ((e = cudaEventRecord(ctx->ev_entry, ctx->stream)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(ctx->s_h2d, ctx->ev_entry, 0)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(ctx->s_comp, ctx->ev_entry, 0)) != cudaSuccess)
    return ordering(e);
  if (ctx->d2h_pending && !chained && (e = cudaStreamWaitEvent(ctx->s_h2d, ctx->ev_d2h[K - 1], 0)) != cudaSuccess)
    return ordering(e);
  for (int k = 0; k < K; ++k) {
    const ew::HostChunk& h = ctx->hchunks[k];
    if (ctx->nfree_valid && (e = cudaStreamWaitEvent(ctx->s_h2d, ctx->ev_nfree[k], 0)) != cudaSuccess)
      return ordering(e);
    if (chained && (e = cudaStreamWaitEvent(ctx->s_h2d, ctx->ev_d2h[k], 0)) != cudaSuccess) return ordering(e);
    if ((e = cudaMemcpyAsync(d_n + h.dof_begin, h_vec_n + h.dof_begin, (size_t)h.n_dofs * sizeof(double),
                             cudaMemcpyHostToDevice, ctx->s_h2d)) != cudaSuccess)
      return cuda_fail(ctx, e, "host to device copy");
    if (split && (rc = split_state(ctx, d_n + h.dof_begin, h.n_dofs, ctx->s_h2d))) return rc;
    if ((e = cudaEventRecord(ctx->ev_in[k], ctx->s_h2d)) != cudaSuccess) return ordering(e);
  }
  // The compute runs on s_comp (the launches go to ctx->stream, swapped for
  // this call).  The last stage that touches d_n (as input, accumulator or
  // output) releases its chunks: chunk k once that stage is done on chunks
  // k-1..k+1 (wavefront), else once it is done everywhere.
  struct StreamSwap {
    ew_ctx* c;
    cudaStream_t saved;
    StreamSwap(ew_ctx* ctx) : c(ctx), saved(ctx->stream) { c->stream = c->s_comp; }
    ~StreamSwap() { c->stream = saved; }
  } swap(ctx);
  int last_n = 0;
  for (int s = 0; s < 5; ++s)
    if (st[s].X == d_n || st[s].A == d_n || st[s].Xout == d_n || st[s].Aout == d_n) last_n = s;
  auto release_all = [&]() -> int {
    for (int k = 0; k < K; ++k)
      if ((e = cudaEventRecord(ctx->ev_nfree[k], ctx->stream)) != cudaSuccess) return ordering(e);
    return EW_OK;
  };
  // copy of chunk k to the host once the last stage has finished it
  auto copy_out = [&](int k) -> int {
    const ew::HostChunk& h = ctx->hchunks[k];
    if ((e = cudaEventRecord(ctx->ev_s5[k], ctx->stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(ctx->s_d2h, ctx->ev_s5[k], 0)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h_vec_np + h.dof_begin, d_np + h.dof_begin, (size_t)h.n_dofs * sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->s_d2h)) != cudaSuccess ||
        (e = cudaEventRecord(ctx->ev_d2h[k], ctx->s_d2h)) != cudaSuccess)
      return cuda_fail(ctx, e, "device to host copy");
    return EW_OK;
  };
  if (staged && ctx->host_wave) {
    // Wavefront: stage s of chunk k is launched on diagonal d = k + 2 s.
    // It reads the previous stage's output on chunks k-1..k+1 (diagonals
    // k + 2 s - 1 and earlier) and overwrites registers that the previous
    // stage read on those chunks, so every dependence points to an earlier
    // diagonal, and the single compute stream runs them in order.  Within a
    // diagonal the first stage, which waits for its input chunks, comes
    // last, so ready work is never queued behind that wait.
    for (int d = 0; d < K + 8; ++d)
      for (int s = 4; s >= 0; --s) {
        const int k = d - 2 * s;
        if (k < 0 || k >= K) continue;
        const ew::HostChunk& h = ctx->hchunks[k];
        if (s == 0)
          for (int j = h.lo; j <= h.hi; ++j)
            if ((e = cudaStreamWaitEvent(ctx->stream, ctx->ev_in[j], 0)) != cudaSuccess) return ordering(e);
        {
          WorkRange wr(ctx, h.item_begin, h.n_items);
          if ((rc = run_stage(ctx, st[s]))) return rc;
        }
        if (s == last_n) {
          // chunk k - 1 is released (its readers are chunks k-2..k), and
          // with the last chunk the last one too
          if (k >= 1 && (e = cudaEventRecord(ctx->ev_nfree[k - 1], ctx->stream)) != cudaSuccess)
            return ordering(e);
          if (k == K - 1 && (e = cudaEventRecord(ctx->ev_nfree[k], ctx->stream)) != cudaSuccess)
            return ordering(e);
        }
        if (s == 4 && (rc = copy_out(k))) return rc;
      }
  } else if (staged) {
    // first stage, chunk by chunk (it writes d_np, which the previous call's
    // copies read: ordered through the input chunks above)
    for (int k = 0; k < K; ++k) {
      const ew::HostChunk& h = ctx->hchunks[k];
      for (int j = h.lo; j <= h.hi; ++j)
        if ((e = cudaStreamWaitEvent(ctx->stream, ctx->ev_in[j], 0)) != cudaSuccess) return ordering(e);
      WorkRange wr(ctx, h.item_begin, h.n_items);
      if ((rc = run_stage(ctx, st[0]))) return rc;
    }
    if (last_n == 0 && (rc = release_all())) return rc;
    for (int s = 1; s < 4; ++s) {
      if ((rc = run_stage(ctx, st[s]))) return rc;
      if (s == last_n && (rc = release_all())) return rc;
    }
    for (int k = 0; k < K; ++k) {
      const ew::HostChunk& h = ctx->hchunks[k];
      {
        WorkRange wr(ctx, h.item_begin, h.n_items);
        if ((rc = run_stage(ctx, st[4]))) return rc;
      }
      if ((rc = copy_out(k))) return rc;
    }
    if (last_n == 4 && (rc = release_all())) return rc;
  } else {
    // the step after every input chunk and after the previous call's output
    // copies (they read d_np, which the step writes)
    if ((e = cudaEventRecord(ctx->ev_h2d, ctx->s_h2d)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(ctx->stream, ctx->ev_h2d, 0)) != cudaSuccess ||
        (ctx->d2h_pending && (e = cudaStreamWaitEvent(ctx->stream, ctx->ev_d2h[K - 1], 0)) != cudaSuccess))
      return ordering(e);
    for (int s = 0; s < 5; ++s)
      if ((rc = run_stage(ctx, st[s]))) return rc;
    if ((rc = release_all())) return rc;
    if ((e = cudaEventRecord(ctx->ev_step, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(ctx->s_d2h, ctx->ev_step, 0)) != cudaSuccess)
      return ordering(e);
    for (int k = 0; k < K; ++k) {
      const ew::HostChunk& h = ctx->hchunks[k];
      if ((e = cudaMemcpyAsync(h_vec_np + h.dof_begin, d_np + h.dof_begin, (size_t)h.n_dofs * sizeof(double),
                               cudaMemcpyDeviceToHost, ctx->s_d2h)) != cudaSuccess ||
          (e = cudaEventRecord(ctx->ev_d2h[k], ctx->s_d2h)) != cudaSuccess)
        return cuda_fail(ctx, e, "device to host copy");
    }
  }
  if ((e = cudaEventRecord(ctx->ev_comp, ctx->stream)) != cudaSuccess) return ordering(e);
  ctx->comp_pending = true;
  ctx->nfree_valid = true;
  ctx->last_host_out = h_vec_np;
  ctx->d2h_pending = true;
  return EW_OK;
}

int ew_wait_host_copies(ew_ctx* ctx) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!ctx->d2h_pending) return EW_OK;
  const cudaError_t e = cudaStreamWaitEvent(ctx->stream, ctx->ev_d2h[ctx->hchunks.size() - 1], 0);
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "host copy ordering");
}

int ew_vec_update(ew_ctx* ctx, double alpha, double* y, double beta, const double* x, double gamma,
                  const double* z) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!y) return fail(ctx, EW_ERR_INVALID, "ew_vec_update: NULL output");
  ew::vec_update_kernel<<<ew::grid_for(ctx->n_dofs), 256, 0, ctx->stream>>>(ctx->n_dofs, alpha, y,
                                                                           beta, x, gamma, z);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "vec_update launch");
}

namespace {
// Coefficients of the low-storage 2-register schemes: a_{s+1,s} (n-1 of
// them) and b_s (n).  LowStorageRK33Reg2 (time_integrators.cc:206-211),
// LowStorageRK59Reg2 (time_integrators.cc:294-311).
struct Lsrk2r {
  int n;
  double a[8];
  double b[9];
};
const Lsrk2r kLsrk33 = {3,
                        {0.755726351946097, 0.386954477304099},
                        {0.245170287303492, 0.184896052186740, 0.569933660509768}};
const Lsrk2r kLsrk59 = {
    9,
    {1107026461565. / 5417078080134., 38141181049399. / 41724347789894.,
     493273079041. / 11940823631197., 1851571280403. / 6147804934346.,
     11782306865191. / 62590030070788., 9452544825720. / 13648368537481.,
     4435885630781. / 26285702406235., 2357909744247. / 11371140753790.},
    {2274579626619. / 23610510767302., 693987741272. / 12394497460941.,
     -347131529483. / 15096185902911., 1144057200723. / 32081666971178.,
     1562491064753. / 11797114684756., 13113619727965. / 44346030145118.,
     393957816125. / 7825732611452., 720647959663. / 6565743875477.,
     3559252274877. / 14424734981077.}};

// Register plan of the fused FP64 stages over three vectors (0 = vec_n,
// 1 = vec_np, 2 = scratch).  Stage 0 reads the state (0) as input and
// accumulator and writes both outputs to 1 and 2; later stages read X (from
// neighbouring cells: never written in the same launch) and A (cell-local:
// one output may overwrite it in place) and write the other output to the
// third vector.  One choice per stage; the plan is the first whose last
// stage leaves the result in vec_np.
struct StagePlan {
  int X, A, Xo, Ao;
};
bool plan_2r(int n, StagePlan* plan) {
  for (int mask = 0; mask < (1 << n); ++mask) {
    int X = 0, A = 0;
    for (int s = 0; s < n; ++s) {
      const bool bit = (mask >> s) & 1;
      StagePlan& p = plan[s];
      p.X = X;
      p.A = A;
      if (s == 0) {
        p.Xo = n == 1 ? -1 : (bit ? 1 : 2);
        p.Ao = n == 1 ? 1 : 3 - (bit ? 1 : 2);
      } else {
        const int F = 3 - X - A;
        if (s + 1 < n) {
          p.Xo = bit ? A : F;
          p.Ao = bit ? F : A;
        } else {
          p.Xo = -1;
          p.Ao = bit ? F : A;
        }
      }
      X = p.Xo;
      A = p.Ao;
    }
    if (plan[n - 1].Ao == 1) return true;
  }
  return false;
}

int lsrk2r_step(ew_ctx* ctx, const Lsrk2r& sc, double dt, double* vec_n, double* vec_np) {
  using namespace ew;
  const int n = sc.n;
  double f1[9], f2[9];
  for (int s = 0; s + 1 < n; ++s) {
    f1[s] = sc.a[s] * dt;
    f2[s] = (sc.b[s] - sc.a[s]) * dt;
  }
  f1[n - 1] = sc.b[n - 1] * dt;
  f2[n - 1] = 0.0;
  int rc;
  if (!ctx->mixed) {
    StagePlan plan[9];
    if (!plan_2r(n, plan)) return fail(ctx, EW_ERR_UNSUPPORTED, "no register plan for the scheme");
    double* R[3] = {vec_n, vec_np, ctx->d_tmp64};
    for (int s = 0; s < n; ++s) {
      const StagePlan& p = plan[s];
      const bool last = s + 1 == n;
      rc = launch_stage(ctx, STAGE_F64, last ? CV_F64_LAST : CV_F64_MID, R[p.A], R[p.X],
                        last ? nullptr : R[p.Xo], R[p.Ao], last ? MODE_RK_LAST : MODE_RK_MID, f1[s],
                        f2[s], 1.0f);
      if (rc) return rc;
    }
    return EW_OK;
  }
  // mixed: the accumulator in vec_np (in place), FP32 stage inputs ping-pong
  float* xb[2] = {ctx->d_x32[0], ctx->d_x32[1]};
  rc = launch_stage(ctx, STAGE_MIX_IN64, CV_MIX_S1, vec_n, vec_n, xb[0], vec_np, MODE_RK_MID, f1[0],
                    f2[0], 1.0f);
  if (rc) return rc;
  int cur = 0;
  for (int s = 1; s < n; ++s) {
    const bool last = s + 1 == n;
    rc = launch_stage(ctx, STAGE_MIX_IN32, last ? CV_MIX_LAST : CV_MIX_MID, vec_np, xb[cur],
                      last ? nullptr : xb[cur ^ 1], vec_np, last ? MODE_RK_LAST : MODE_RK_MID, f1[s],
                      f2[s], 1.0f);
    if (rc) return rc;
    cur ^= 1;
  }
  return EW_OK;
}
}  // namespace

int ew_lsrk_step(ew_ctx* ctx, int32_t scheme, double dt, double* vec_n, double* vec_np) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!vec_n || !vec_np || vec_n == vec_np)
    return fail(ctx, EW_ERR_INVALID, "ew_lsrk_step: vec_n and vec_np must be distinct");
  switch (scheme) {
    case EW_LSRK33R2: return lsrk2r_step(ctx, kLsrk33, dt, vec_n, vec_np);
    case EW_LSRK45R2: return ew_lsrk45_step(ctx, dt, vec_n, vec_np);
    case EW_LSRK59R2: return lsrk2r_step(ctx, kLsrk59, dt, vec_n, vec_np);
    default: return fail(ctx, EW_ERR_INVALID, "ew_lsrk_step: unknown scheme");
  }
}

int ew_lsrk45_steps(ew_ctx* ctx, double dt, int64_t n_steps, double* vec_n, double* vec_np) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!vec_n || !vec_np || vec_n == vec_np || n_steps < 0)
    return fail(ctx, EW_ERR_INVALID, "ew_lsrk45_steps: invalid vectors or step count");
  if (n_steps == 0)
    return cudaMemcpyAsync(vec_np, vec_n, (size_t)ctx->n_dofs * sizeof(double),
                           cudaMemcpyDeviceToDevice, ctx->stream) == cudaSuccess
               ? EW_OK
               : fail(ctx, EW_ERR_CUDA, "ew_lsrk45_steps: copy");
  using namespace ew;
  if (ctx->ff && ctx->line) {
    // Compensated, Cartesian.  Between two steps the state is kept as float
    // pairs (8 bytes, like FP64): the last stage of every step but the call's
    // final one writes the pairs in place of its accumulator, and the next
    // step's first stage reads them as its input and accumulator at once, with
    // its own accumulator in the other vector.  State and accumulator trade
    // vectors every step; the call's final step writes FP64.
    const double f1[5] = {kA21 * dt, kA32 * dt, kA43 * dt, kA54 * dt, kB5 * dt};
    const double f2[5] = {(kB1 - kA21) * dt, (kB2 - kA32) * dt, (kB3 - kA43) * dt,
                          (kB4 - kA54) * dt, 0.0};
    float* xb[2] = {ctx->d_x32[0], ctx->d_x32[1]};
    double* st = vec_n;   // state: FP64 before the first step, float pairs after
    double* ac = vec_np;  // accumulator of the current step
    for (int64_t step = 0; step < n_steps; ++step) {
      const bool last_step = step + 1 == n_steps;
      if (step == 0) {
        // the FP64 state split in place into float pairs: then like any step
        if ((rc = split_state(ctx, st, ctx->n_dofs, ctx->stream))) return rc;
        rc = launch_stage(ctx, STAGE_MIX_IN32, CV_MIX_MID, st, st, xb[0], ac, MODE_RK_MID, f1[0], f2[0],
                          1.0f);
      } else
        rc = launch_stage(ctx, STAGE_MIX_IN32, CV_MIX_MID, st, st, xb[0], ac, MODE_RK_MID, f1[0],
                          f2[0], 1.0f);
      if (rc) return rc;
      int cur = 0;
      for (int s = 1; s < 4; ++s) {
        rc = launch_stage(ctx, STAGE_MIX_IN32, CV_MIX_MID, ac, xb[cur], xb[cur ^ 1], ac, MODE_RK_MID,
                          f1[s], f2[s], 1.0f);
        if (rc) return rc;
        cur ^= 1;
      }
      rc = launch_stage(ctx, STAGE_MIX_IN32, last_step ? CV_MIX_LAST : CV_FF_LAST_PAIR, ac, xb[cur],
                        nullptr, ac, MODE_RK_LAST, f1[4], f2[4], 1.0f);
      if (rc) return rc;
      std::swap(st, ac);
    }
    if (st != vec_np &&
        cudaMemcpyAsync(vec_np, st, (size_t)ctx->n_dofs * sizeof(double), cudaMemcpyDeviceToDevice,
                        ctx->stream) != cudaSuccess)
      return fail(ctx, EW_ERR_CUDA, "ew_lsrk45_steps: copy");
    return EW_OK;
  }
  if (!ctx->mixed || !ctx->line) {
    // one step at a time; the state alternates between the two vectors
    double* a = vec_n;
    double* b = vec_np;
    for (int64_t s = 0; s < n_steps; ++s) {
      if ((rc = ew_lsrk45_step(ctx, dt, a, b))) return rc;
      std::swap(a, b);
    }
    if (a != vec_np &&
        cudaMemcpyAsync(vec_np, a, (size_t)ctx->n_dofs * sizeof(double), cudaMemcpyDeviceToDevice,
                        ctx->stream) != cudaSuccess)
      return fail(ctx, EW_ERR_CUDA, "ew_lsrk45_steps: copy");
    return EW_OK;
  }
  // Mixed, Cartesian.  The accumulator lives in vec_np.  Between two steps
  // the state is a float pair held as two FP32 arrays: hi in the stage
  // input buffer the last stage does not read, lo in vec_n's memory (free
  // once the call's first stage has read the FP64 input).  The next first
  // stage reads hi like a middle stage reads its input; the call's final
  // step writes FP64 to vec_np.
  const double f1[5] = {kA21 * dt, kA32 * dt, kA43 * dt, kA54 * dt, kB5 * dt};
  const double f2[5] = {(kB1 - kA21) * dt, (kB2 - kA32) * dt, (kB3 - kA43) * dt, (kB4 - kA54) * dt,
                        0.0};
  float* xb[2] = {ctx->d_x32[0], ctx->d_x32[1]};
  float* lo = reinterpret_cast<float*>(vec_n);
  int hi = -1;  // stage-input buffer holding the state's hi part
  for (int64_t step = 0; step < n_steps; ++step) {
    const bool last_step = step + 1 == n_steps;
    int cur;  // buffer of the next stage input
    if (step == 0) {
      cur = 0;
      rc = launch_stage(ctx, STAGE_MIX_IN64, CV_MIX_S1, vec_n, vec_n, xb[cur], vec_np, MODE_RK_MID,
                        f1[0], f2[0], 1.0f);
    } else {
      cur = hi ^ 1;
      rc = launch_stage(ctx, STAGE_MIX_IN32, CV_MIX_S1_FF, reinterpret_cast<const double*>(lo), xb[hi],
                        xb[cur], vec_np, MODE_RK_MID, f1[0], f2[0], 1.0f);
    }
    if (rc) return rc;
    for (int s = 1; s < 5; ++s) {
      if (s < 4) {
        rc = launch_stage(ctx, STAGE_MIX_IN32, CV_MIX_MID, vec_np, xb[cur], xb[cur ^ 1], vec_np,
                          MODE_RK_MID, f1[s], f2[s], 1.0f);
        cur ^= 1;
      } else if (last_step) {
        rc = launch_stage(ctx, STAGE_MIX_IN32, CV_MIX_LAST, vec_np, xb[cur], nullptr, vec_np,
                          MODE_RK_LAST, f1[s], f2[s], 1.0f);
      } else {
        rc = launch_stage(ctx, STAGE_MIX_IN32, CV_MIX_LAST_FF, vec_np, xb[cur], xb[cur ^ 1],
                          reinterpret_cast<double*>(lo), MODE_RK_LAST, f1[s], f2[s], 1.0f);
        hi = cur ^ 1;
      }
      if (rc) return rc;
    }
  }
  return EW_OK;
}

// ---- LSRK45 step with its scratch in a static device array ------------------
namespace {
// Stage scratch of ew_lsrk45_step_static (two FP32 stage inputs, or the FP64
// third register); held by every device that loads the library.
__device__ __align__(256) float g_static_scratch[EW_STATIC_SCRATCH_BYTES / sizeof(float)];
constexpr int kMaxDevices = 64;
float* g_static_ptr[kMaxDevices] = {};
std::mutex g_static_mutex;

// Device address of the array on the current device (looked up once per device).
int static_scratch(ew_ctx* c, float** out) {
  std::lock_guard<std::mutex> lk(g_static_mutex);
  if (c->device < 0 || c->device >= kMaxDevices)
    return fail(c, EW_ERR_INVALID, "device ordinal too large for the static scratch table");
  if (!g_static_ptr[c->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(c, e, "cudaGetSymbolAddress(static scratch)");
    g_static_ptr[c->device] = static_cast<float*>(p);
  }
  *out = g_static_ptr[c->device];
  return EW_OK;
}
}  // namespace

int ew_lsrk45_step_static(ew_ctx* ctx, double dt, double* vec_n, double* vec_np) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!vec_n || !vec_np || vec_n == vec_np)
    return fail(ctx, EW_ERR_INVALID, "ew_lsrk45_step_static: vec_n and vec_np must be distinct");
  if (ctx->ff)
    return fail(ctx, EW_ERR_UNSUPPORTED,
                "ew_lsrk45_step_static: not built for EW_PREC_MIXED_FF (its stage inputs are float "
                "pairs, twice the static scratch)");
  if (ctx->n_dofs > EW_STATIC_SCRATCH_MAX_DOFS)
    return fail(ctx, EW_ERR_TOO_LARGE,
                "ew_lsrk45_step_static: " + std::to_string(ctx->n_dofs) +
                    " DoFs exceed the static scratch (at most " +
                    std::to_string((long long)EW_STATIC_SCRATCH_MAX_DOFS) + " DoFs)");
  float* scratch = nullptr;
  if ((rc = static_scratch(ctx, &scratch))) return rc;
  // FP64: the third register of the two-register scheme lives in the array;
  // mixed: the two FP32 stage inputs (the second at a 256-byte aligned offset)
  const size_t off = ((size_t)ctx->n_dofs + 63) & ~(size_t)63;
  return lsrk45_stages(ctx, dt, vec_n, vec_np, reinterpret_cast<double*>(scratch), scratch,
                       scratch + off);
}

int ew_apply_ader(ew_ctx* ctx, double dt, const double* src, double* dst) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!src || !dst || src == dst) return fail(ctx, EW_ERR_INVALID, "ew_apply_ader: src/dst invalid");
  void* T = ctx->mixed ? static_cast<void*>(ctx->d_x32[0]) : static_cast<void*>(ctx->d_tmp64);
  if ((rc = launch_ck(ctx, dt, src, T))) return rc;
  const int var = ctx->mixed ? ew::STAGE_MIX_IN32 : ew::STAGE_F64;
  const int cv = ctx->mixed ? ew::CV_MIX_APPLY32 : ew::CV_F64_APPLY;
  return launch_stage(ctx, var, cv, nullptr, T, nullptr, dst, ew::MODE_APPLY, 0.0, 0.0, -1.0f);
}

int ew_aderadconfull_step(ew_ctx* ctx, double dt, const double* vec_n, double* vec_np) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!vec_n || !vec_np || vec_n == vec_np)
    return fail(ctx, EW_ERR_INVALID, "ew_aderadconfull_step: vec_n and vec_np must be distinct");
  // w_0 = u, w_{j+1} = M^-1 A(w_j); u' = u + dt w_1 + sum_{j=1..k} fac_j (-1)^j w_{j+1}
  // with fac_1 = -dt^2/2, fac_{j+1} = -fac_j dt / (j + 2): the reference's
  // series (its intermediate vectors are -(previous result)), signs folded
  // into the coefficients
  for (int i = 0; i < 2; ++i)
    if (!ctx->d_ad[i] && (rc = dev_alloc(ctx, &ctx->d_ad[i], (size_t)ctx->n_dofs))) return rc;
  cudaError_t e = cudaMemcpyAsync(vec_np, vec_n, (size_t)ctx->n_dofs * 8, cudaMemcpyDeviceToDevice,
                                  ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "copy");
  const int var = ctx->mixed ? ew::STAGE_MIX_IN64 : ew::STAGE_F64;
  const int cv = ctx->mixed ? ew::CV_MIX_APPLY64 : ew::CV_F64_APPLY;
  double fac = -0.5 * dt * dt;
  for (int j = 0; j <= ctx->degree; ++j) {
    const double* in = j == 0 ? vec_n : ctx->d_ad[(j - 1) & 1];
    double* out = ctx->d_ad[j & 1];
    if ((rc = launch_stage(ctx, var, cv, nullptr, in, nullptr, out, ew::MODE_APPLY, 0.0, 0.0, 1.0f)))
      return rc;
    double c = dt;
    if (j > 0) {
      c = (j & 1) ? -fac : fac;
      fac *= -dt / (j + 2);
    }
    ew::axpy_kernel<<<ew::grid_for(ctx->n_dofs), 256, 0, ctx->stream>>>(ctx->n_dofs, c, out, vec_np);
    ++ctx->launches;
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, e, "axpy launch");
  }
  return EW_OK;
}

int ew_ader_step(ew_ctx* ctx, double dt, const double* vec_n, double* vec_np) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!vec_n || !vec_np || vec_n == vec_np)
    return fail(ctx, EW_ERR_INVALID, "ew_ader_step: vec_n and vec_np must be distinct");
  void* T = ctx->mixed ? static_cast<void*>(ctx->d_x32[0]) : static_cast<void*>(ctx->d_tmp64);
  if ((rc = launch_ck(ctx, dt, vec_n, T))) return rc;
  const int var = ctx->mixed ? ew::STAGE_MIX_IN32 : ew::STAGE_F64;
  const int cv = ctx->mixed ? ew::CV_MIX_UPD : ew::CV_F64_LAST;
  // vec_np = vec_n - (-M^{-1}A(T)) = vec_n + M^{-1}A(T)
  return launch_stage(ctx, var, cv, vec_n, T, nullptr, vec_np, ew::MODE_RK_LAST, 1.0, 0.0, 1.0f);
}

int ew_quadrature_points(ew_ctx* ctx, double* xyz) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!xyz) return fail(ctx, EW_ERR_INVALID, "NULL output");
  ew::qpoints_kernel<<<ew::grid_for(ctx->n_cells * ctx->N), 256, 0, ctx->stream>>>(
      ctx->d_verts, ctx->n_cells, ctx->dim, ctx->np, ctx->d_nodes, xyz);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "qpoints launch");
}

static int make_modes(ew_ctx* ctx, int32_t n_modes, const double* amp, const int32_t* kvec,
                      ew::Modes* ms) {
  if (n_modes < 0 || n_modes > ew::kMaxModes || (n_modes > 0 && (!amp || !kvec)))
    return fail(ctx, EW_ERR_INVALID, "membrane modes: 0..8 modes with amplitudes and wave numbers");
  std::memset(ms, 0, sizeof(*ms));
  ms->n = n_modes;
  for (int m = 0; m < n_modes; ++m) {
    ms->amp[m] = amp[m];
    bool nz = false;
    for (int d = 0; d < 3; ++d) {
      ms->k[m][d] = kvec[3 * m + d];
      if (d < ctx->dim && kvec[3 * m + d] != 0) nz = true;
    }
    if (!nz) return fail(ctx, EW_ERR_INVALID, "membrane mode with zero wave vector");
  }
  return EW_OK;
}

int ew_project_membrane(ew_ctx* ctx, int32_t n_modes, const double* amp, const int32_t* kvec,
                        double t, double* u) {
  int rc = check(ctx);
  if (rc) return rc;
  ew::Modes ms;
  if ((rc = make_modes(ctx, n_modes, amp, kvec, &ms))) return rc;
  if (!u) return fail(ctx, EW_ERR_INVALID, "NULL output");
  ew::project_membrane_kernel<<<ew::grid_for(ctx->n_cells * ctx->N), 256, 0, ctx->stream>>>(
      ctx->d_verts, ctx->n_cells, ctx->dim, ctx->np, ctx->d_nodes, ms, t, u);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "project launch");
}

int ew_project_gaussian(ew_ctx* ctx, const double* x0, double width, double amp, double* u) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!x0 || !u || !(width > 0.0)) return fail(ctx, EW_ERR_INVALID, "gaussian: bad arguments");
  ew::project_gaussian_kernel<<<ew::grid_for(ctx->n_cells * ctx->N), 256, 0, ctx->stream>>>(
      ctx->d_verts, ctx->n_cells, ctx->dim, ctx->np, ctx->d_nodes, x0[0], ctx->dim > 1 ? x0[1] : 0.0,
      ctx->dim > 2 ? x0[2] : 0.0, width, amp, u);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "project launch");
}

static int run_l2(ew_ctx* ctx, const double* a, const double* b, const ew::Modes& ms, double t,
                  int mode, double* out) {
  cudaError_t e = cudaMemsetAsync(ctx->d_acc, 0, 4 * sizeof(double), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "memset");
  const int m = ctx->l2_m;
  int M = 1;
  for (int d = 0; d < ctx->dim; ++d) M *= m;
  const int grid = (int)std::min<int64_t>(ew::grid_for(ctx->n_cells * M), 8 * ctx->num_sms);
  ew::l2_kernel<<<grid, 256, 0, ctx->stream>>>(ctx->d_verts, ctx->n_cells, ctx->dim, ctx->np, m,
                                               ctx->d_l2, ctx->d_l2 + m * ctx->np,
                                               ctx->d_l2 + m * ctx->np + m, a, b, ms, t, mode,
                                               ctx->d_acc);
  ++ctx->launches;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "l2 launch");
  double h[4];
  e = cudaMemcpyAsync(h, ctx->d_acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "l2 readback");
  out[0] = std::sqrt(h[0]);
  out[1] = std::sqrt(h[1]);
  out[2] = std::sqrt(h[2]);
  return EW_OK;
}

int ew_l2_errors_membrane(ew_ctx* ctx, const double* u, int32_t n_modes, const double* amp,
                          const int32_t* kvec, double t, double out[3]) {
  int rc = check(ctx);
  if (rc) return rc;
  ew::Modes ms;
  if ((rc = make_modes(ctx, n_modes, amp, kvec, &ms))) return rc;
  if (!u || !out) return fail(ctx, EW_ERR_INVALID, "NULL argument");
  return run_l2(ctx, u, nullptr, ms, t, 0, out);
}

int ew_l2_difference(ew_ctx* ctx, const double* a, const double* b, double out[2]) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!a || !b || !out) return fail(ctx, EW_ERR_INVALID, "NULL argument");
  ew::Modes ms;
  std::memset(&ms, 0, sizeof(ms));
  double o3[3];
  rc = run_l2(ctx, a, b, ms, 0.0, 1, o3);
  out[0] = o3[0];
  out[1] = o3[1];
  return rc;
}

int ew_tune_set(int32_t dim, int32_t degree, int32_t precision, int32_t cells_per_block) {
  if (dim < 2 || dim > 3 || degree < 1 || degree > EW_MAX_DEGREE || precision < 0 ||
      precision > 2 || cells_per_block < 0 || cells_per_block > 1024)
    return EW_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ew::g_tuned_mutex);
  ew::g_tuned[dim - 2][degree][precision] = cells_per_block;
  return EW_OK;
}

int32_t ew_tune_get(int32_t dim, int32_t degree, int32_t precision) {
  return ew::tuned_cells_per_block(dim, degree, precision);
}

int ew_tune_set_staging(int32_t dim, int32_t degree, int32_t precision, int32_t nb_staging) {
  if (dim < 2 || dim > 3 || degree < 1 || degree > EW_MAX_DEGREE || precision < 0 ||
      precision > 2 || nb_staging < 0 || nb_staging > 2)
    return EW_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ew::g_tuned_mutex);
  ew::g_tuned_staging[dim - 2][degree][precision] = nb_staging;
  return EW_OK;
}

int32_t ew_tune_get_staging(int32_t dim, int32_t degree, int32_t precision) {
  return ew::tuned_staging(dim, degree, precision);
}

int ew_set_receivers(ew_ctx* ctx, int32_t n, const double* points) {
  int rc = check(ctx);
  if (rc) return rc;
  if (n < 0 || (n > 0 && !points)) return fail(ctx, EW_ERR_INVALID, "ew_set_receivers: invalid points");
  const int dim = ctx->dim, nv = 1 << dim, N = ctx->N;
  std::vector<double> verts((size_t)ctx->n_cells * nv * dim);
  cudaError_t e = cudaMemcpy(verts.data(), ctx->d_verts, verts.size() * 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "vertex readback");
  const ew::GaussRule g = ew::gauss_rule(ctx->np);
  std::vector<int32_t> cells(std::max(n, 1), 0);
  std::vector<double> w((size_t)std::max(n, 1) * N, 0.0);
  for (int r = 0; r < n; ++r) {
    const double* p = points + (size_t)r * dim;
    int32_t found = -1;
    double xi[3] = {0, 0, 0};
    for (int64_t c = 0; c < ctx->n_cells && found < 0; ++c) {
      const double* V = verts.data() + (size_t)c * nv * dim;
      bool inbox = true;
      for (int d = 0; d < dim && inbox; ++d) {
        double lo = V[d], hi = V[d];
        for (int v = 1; v < nv; ++v) {
          lo = std::min(lo, V[v * dim + d]);
          hi = std::max(hi, V[v * dim + d]);
        }
        const double tol = 1e-10 * (hi - lo);
        inbox = p[d] >= lo - tol && p[d] <= hi + tol;
      }
      if (inbox && invert_map(dim, V, p, xi)) found = (int32_t)c;
    }
    if (found < 0) return fail(ctx, EW_ERR_INVALID, "ew_set_receivers: point " + std::to_string(r) + " is outside the mesh");
    cells[r] = found;
    for (int q = 0; q < N; ++q) {
      double v = 1.0;
      int t = q;
      for (int d = 0; d < dim; ++d) {
        v *= ew::lagrange(g.x, t % ctx->np, std::min(1.0, std::max(0.0, xi[d])));
        t /= ctx->np;
      }
      w[(size_t)r * N + q] = v;
    }
  }
  if (ctx->d_rec_cell) cudaFree(ctx->d_rec_cell);
  if (ctx->d_rec_w) cudaFree(ctx->d_rec_w);
  ctx->d_rec_cell = nullptr;
  ctx->d_rec_w = nullptr;
  ctx->n_rec = 0;
  if ((rc = dev_alloc(ctx, &ctx->d_rec_cell, cells.size())) || (rc = dev_alloc(ctx, &ctx->d_rec_w, w.size())) ||
      (rc = upload(ctx, ctx->d_rec_cell, cells.data(), cells.size() * 4)) ||
      (rc = upload(ctx, ctx->d_rec_w, w.data(), w.size() * 8)))
    return rc;
  ctx->n_rec = n;
  return EW_OK;
}

int ew_sample_receivers(ew_ctx* ctx, const double* state, double* out) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!state || !out) return fail(ctx, EW_ERR_INVALID, "ew_sample_receivers: NULL vector");
  if (ctx->n_rec == 0) return EW_OK;
  const int threads = 256, per_block = threads / 32;
  receivers_kernel<<<(ctx->n_rec + per_block - 1) / per_block, threads, 0, ctx->stream>>>(
      state, ctx->n_rec, ctx->F, ctx->N, ctx->d_rec_cell, ctx->d_rec_w, out);
  ++ctx->launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EW_OK : cuda_fail(ctx, e, "receiver launch");
}

int ew_l2_error_post_membrane(ew_ctx* ctx, const double* state, int32_t n_modes,
                               const double* amps, const int32_t* kvecs, double t, double* out) {
  int rc = check(ctx);
  if (rc) return rc;
  if (!state || !out) return fail(ctx, EW_ERR_INVALID, "ew_l2_error_post_membrane: NULL argument");
  ew::Modes ms;
  if ((rc = make_modes(ctx, n_modes, amps, kvecs, &ms))) return rc;
  const int dim = ctx->dim, np = ctx->np, m = np + 1, me = m + 1;
  int Mp = 1;
  for (int d = 0; d < dim; ++d) Mp *= m;
  if (Mp > 1024)
    return fail(ctx, EW_ERR_UNSUPPORTED,
                "ew_l2_error_post_membrane: one thread per QGauss(k+2) point, at most 1024 (3-D degree <= 8)");
  if (!ctx->d_post) {
    // interp (m x np), qx, qw, D (m x m), Ie (me x m), ex, ew
    const ew::GaussRule g = ew::gauss_rule(np), gp = ew::gauss_rule(m), ge = ew::gauss_rule(me);
    std::vector<double> pb;
    for (int a = 0; a < m; ++a)
      for (int i = 0; i < np; ++i) pb.push_back(ew::lagrange(g.x, i, gp.x[a]));
    pb.insert(pb.end(), gp.x.begin(), gp.x.end());
    pb.insert(pb.end(), gp.w.begin(), gp.w.end());
    for (int a = 0; a < m; ++a)
      for (int j = 0; j < m; ++j) pb.push_back(ew::lagrange_deriv(gp.x, j, gp.x[a]));
    for (int a = 0; a < me; ++a)
      for (int j = 0; j < m; ++j) pb.push_back(ew::lagrange(gp.x, j, ge.x[a]));
    pb.insert(pb.end(), ge.x.begin(), ge.x.end());
    pb.insert(pb.end(), ge.w.begin(), ge.w.end());
    if ((rc = dev_alloc(ctx, &ctx->d_post, pb.size())) ||
        (rc = upload(ctx, ctx->d_post, pb.data(), pb.size() * 8)))
      return rc;
  }
  if (!ctx->d_ad[0] && (rc = dev_alloc(ctx, &ctx->d_ad[0], (size_t)ctx->n_dofs))) return rc;
  // du/dt = M^-1 A(u) (its velocity part feeds the right-hand side)
  const int var = ctx->mixed ? ew::STAGE_MIX_IN64 : ew::STAGE_F64;
  const int cv = ctx->mixed ? ew::CV_MIX_APPLY64 : ew::CV_F64_APPLY;
  if ((rc = launch_stage(ctx, var, cv, nullptr, state, nullptr, ctx->d_ad[0], ew::MODE_APPLY, 0.0,
                         0.0, 1.0f)))
    return rc;
  cudaError_t e = cudaMemsetAsync(ctx->d_acc, 0, 4 * sizeof(double), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "memset");
  const size_t smem = ((size_t)12 * Mp + 33) * sizeof(double);
  if (smem > 48 * 1024 &&
      (e = cudaFuncSetAttribute(ew::post_pressure_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem)) != cudaSuccess)
    return cuda_fail(ctx, e, "post kernel attribute");
  ew::post_pressure_kernel<<<(unsigned)ctx->n_cells, (Mp + 31) / 32 * 32, smem, ctx->stream>>>(
      ctx->d_verts, ctx->d_mat, ctx->ff ? 2 : (ctx->mixed ? 0 : 1), dim, np, ctx->d_post, state, ctx->d_ad[0], ms, t,
      ctx->d_acc);
  ++ctx->launches;
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, e, "post kernel launch");
  double h[4];
  e = cudaMemcpyAsync(h, ctx->d_acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "post readback");
  *out = std::sqrt(h[3]);
  return EW_OK;
}

int ew_synchronize(ew_ctx* ctx) {
  int rc = check(ctx);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "stream synchronize");
  if (ctx->s_d2h && (e = cudaStreamSynchronize(ctx->s_d2h)) != cudaSuccess)
    return cuda_fail(ctx, e, "host copy stream synchronize");
  int flags = 0;
  e = cudaMemcpy(&flags, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "error flag readback");
  if (flags) {
    std::string m = "device error flag";
    if (flags & ew::ERR_BAD_NEIGHBOR) m += ": neighbor index out of range";
    if (flags & ew::ERR_BAD_BOUNDARY_ID) m += ": invalid boundary id";
    if (flags & ew::ERR_BAD_LAUNCH) m += ": launch shape mismatch";
    if (flags & 8) m += ": wait for a bulk copy timed out";
    cudaMemset(ctx->d_err, 0, sizeof(int));
    return fail(ctx, EW_ERR_DEVICE, m);
  }
  return EW_OK;
}

int ew_check_wait_timeout(ew_ctx* ctx, int32_t polls) {
  int rc = check(ctx);
  if (rc) return rc;
  if (polls < 1) return fail(ctx, EW_ERR_INVALID, "ew_check_wait_timeout: polls must be positive");
  // earlier work first, so that its flags are not mistaken for this one's
  if ((rc = ew_synchronize(ctx))) return rc;
  cudaError_t e = ew::launch_wait_timeout(polls, ctx->d_err, ctx->stream);
  ++ctx->launches;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "wait time-out launch");
  return ew_synchronize(ctx);
}

}  // extern "C"
