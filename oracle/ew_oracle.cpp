// ew_oracle.cpp -- CPU oracle for the ExWave explicit DG hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain FP64 C++, the
// arithmetic that ExWave (kronbichler/exwave) performs through deal.II's
// MatrixFree on its hot path, so that the CUDA kernels of exwave_gb300 can be
// checked against it.  Only the test-suite, the smoke check and the CPU
// baseline leg of the benchmark load it; the product library never does.
//
// Parity is pinned against the reference's own regression outputs
// (tests/*.output of the reference): the oracle reproduces their "error p",
// "error v" and "solution mag p" columns at the printed precision (see
// tests/test_oracle_golden.py).
//
// Discretisation (re-derived, not ported): the DG space Q_k with Gauss
// quadrature of k+1 points is represented in the Lagrange basis collocated at
// those Gauss points.  The discrete solution is a property of the space and
// the quadrature, not of the basis, so results agree with the reference's
// FE_DGQ(k) basis up to round-off:
//   * the mass matrix with the same quadrature is diagonal (JxW), which is
//     what CellwiseInverseMassMatrix inverts (wave_equation_operations.cc:633-661);
//   * the L2 projection of the initial field with QGauss(k+1)
//     (wave_equation_operations.cc:902-935) is point sampling.
//
// Layout of every state vector: [cell][field][point], fields u_0..u_{d-1}, p,
// points lexicographic with x fastest; cells in the order of the mesh arrays.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kMaxDim = 3;

// ---------------------------------------------------------------- quadrature
// Gauss-Legendre rule with n points on [0,1] (weights sum to one), Newton
// iteration on the Legendre polynomial; nodes are mirrored so that
// x[n-1-i] = 1 - x[i] holds exactly (same convention as QGauss<1>).
struct Rule {
  int n = 0;
  std::vector<double> x, w;
};

Rule gauss_rule(int n) {
  Rule r;
  r.n = n;
  r.x.assign(n, 0.0);
  r.w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double t = std::cos(kPi * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) {
        p1 = t;
        p0 = 1.0;
      }
      dp = (n == 1) ? 1.0 : n * (t * p1 - p0) / (t * t - 1.0);
      const double dt = p1 / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-17) break;
    }
    {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = (n == 1) ? 1.0 : n * (t * p1 - p0) / (t * t - 1.0);
    }
    const double w = 2.0 / ((1.0 - t * t) * dp * dp);
    // t is descending in i; x = (1 - t)/2 is ascending.
    r.x[i] = 0.5 * (1.0 - t);
    r.x[n - 1 - i] = 0.5 * (1.0 + t);
    r.w[i] = 0.5 * w;
    r.w[n - 1 - i] = 0.5 * w;
  }
  if (n % 2 == 1) r.x[n / 2] = 0.5;
  return r;
}

// Lagrange basis on a set of nodes.
struct Lagrange {
  std::vector<double> y;  // nodes
  double value(int j, double x) const {
    double v = 1.0;
    for (size_t m = 0; m < y.size(); ++m)
      if ((int)m != j) v *= (x - y[m]) / (y[j] - y[m]);
    return v;
  }
  double deriv(int j, double x) const {
    double s = 0.0;
    for (size_t m = 0; m < y.size(); ++m) {
      if ((int)m == j) continue;
      double prod = 1.0 / (y[j] - y[m]);
      for (size_t r = 0; r < y.size(); ++r)
        if ((int)r != j && r != m) prod *= (x - y[r]) / (y[j] - y[r]);
      s += prod;
    }
    return s;
  }
};

// One-dimensional collocation data for n Gauss points.
struct Basis1D {
  int n = 0;
  Rule rule;
  Lagrange lag;
  std::vector<double> D;   // D[i*n+j] = l_j'(x_i)
  std::vector<double> L0;  // l_j(0)
  std::vector<double> L1;  // l_j(1)
  explicit Basis1D(int n_ = 1) { init(n_); }
  void init(int n_) {
    n = n_;
    rule = gauss_rule(n);
    lag.y = rule.x;
    D.assign(n * n, 0.0);
    L0.assign(n, 0.0);
    L1.assign(n, 0.0);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) D[i * n + j] = lag.deriv(j, rule.x[i]);
    for (int j = 0; j < n; ++j) {
      L0[j] = lag.value(j, 0.0);
      L1[j] = lag.value(j, 1.0);
    }
  }
};

int ipow(int b, int e) {
  int r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

// ---------------------------------------------------------------- geometry
// Multilinear map of a cell from its 2^dim vertices (deal.II lexicographic
// vertex order, bit e of the vertex number selects the upper end in
// direction e).  With a flat manifold, MappingQGeneric(k) interpolates this
// map exactly (explicit_wave.cc:161, input_parameters.h:66-68).
void map_point(int dim, const double* V, const double* xi, double* x) {
  const int nv = 1 << dim;
  for (int i = 0; i < dim; ++i) x[i] = 0.0;
  for (int v = 0; v < nv; ++v) {
    double phi = 1.0;
    for (int e = 0; e < dim; ++e) phi *= ((v >> e) & 1) ? xi[e] : 1.0 - xi[e];
    for (int i = 0; i < dim; ++i) x[i] += V[v * dim + i] * phi;
  }
}

// J[i][j] = d x_i / d xi_j
void jacobian(int dim, const double* V, const double* xi, double J[3][3]) {
  const int nv = 1 << dim;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J[i][j] = (i == j && i >= dim) ? 1.0 : 0.0;
  for (int v = 0; v < nv; ++v) {
    for (int j = 0; j < dim; ++j) {
      double dphi = ((v >> j) & 1) ? 1.0 : -1.0;
      for (int e = 0; e < dim; ++e)
        if (e != j) dphi *= ((v >> e) & 1) ? xi[e] : 1.0 - xi[e];
      for (int i = 0; i < dim; ++i) J[i][j] += V[v * dim + i] * dphi;
    }
  }
}

// Inverse transpose: JiT[d][e] = d xi_e / d x_d (what FEEvaluation applies to
// reference gradients).
double inverse_transpose(int dim, const double J[3][3], double JiT[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) JiT[i][j] = 0.0;
  if (dim == 2) {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double id = 1.0 / det;
    // J^{-1} = [ J11 -J01; -J10 J00 ] / det ; JiT = (J^{-1})^T
    JiT[0][0] = J[1][1] * id;
    JiT[0][1] = -J[1][0] * id;
    JiT[1][0] = -J[0][1] * id;
    JiT[1][1] = J[0][0] * id;
    return det;
  }
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double c10 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  const double c11 = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  const double c12 = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  const double c20 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  const double c21 = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  const double c22 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double id = 1.0 / det;
  // cofactor matrix C[i][j]; J^{-1} = C^T/det, so JiT = C/det
  JiT[0][0] = c00 * id; JiT[0][1] = c01 * id; JiT[0][2] = c02 * id;
  JiT[1][0] = c10 * id; JiT[1][1] = c11 * id; JiT[1][2] = c12 * id;
  JiT[2][0] = c20 * id; JiT[2][1] = c21 * id; JiT[2][2] = c22 * id;
  return det;
}

// ---------------------------------------------------------------- mesh
struct Mesh {
  int dim = 2;
  int64_t n_cells = 0;
  std::vector<double> vert;     // [cell][vertex][dim]
  std::vector<int32_t> nbr;     // [cell][2*dim]; <0: boundary id = -value
  std::vector<double> speed;    // [cell]
  std::vector<double> density;  // [cell]
};

// subdivided_hyper_cube(n_intervals) on [0,1]^dim, the reference's vertex
// transform x_0 += f * prod_d sin(pi x_d) (input_parameters.h:42-50,66-68),
// then n_refinements global refinements with a flat manifold, which places
// the new vertices on the multilinear map of each coarse cell.  Cells are
// numbered lexicographically on the fine grid (x fastest).  All boundary
// faces get the same id (input_parameters.h:72-76), one material with c=rho=1
// (input_parameters.cc:22-29).
Mesh hypercube_mesh(int dim, int n_int, int n_ref, double f, int bid) {
  Mesh m;
  m.dim = dim;
  const int sub = 1 << n_ref;
  const int M = n_int * sub;
  const int nv_c = n_int + 1;
  // transformed coarse vertices
  std::vector<double> cv((size_t)ipow(nv_c, dim) * dim);
  for (int64_t idx = 0; idx < ipow(nv_c, dim); ++idx) {
    int64_t t = idx;
    double p[3] = {0, 0, 0};
    for (int e = 0; e < dim; ++e) {
      p[e] = (double)(t % nv_c) / n_int;
      t /= nv_c;
    }
    double s = f;
    for (int e = 0; e < dim; ++e) s *= std::sin(kPi * p[e]);
    p[0] = p[0] + s;
    for (int e = 0; e < dim; ++e) cv[idx * dim + e] = p[e];
  }
  auto fine_vertex = [&](const int* g, double* out) {
    // g: fine grid vertex index per direction
    int cc[3], loc[3];
    double xi[3];
    for (int e = 0; e < dim; ++e) {
      cc[e] = std::min(g[e] / sub, n_int - 1);
      loc[e] = g[e] - cc[e] * sub;
      xi[e] = (double)loc[e] / sub;
    }
    double V[8 * 3];
    for (int v = 0; v < (1 << dim); ++v) {
      int64_t idx = 0, str = 1;
      for (int e = 0; e < dim; ++e) {
        idx += (cc[e] + ((v >> e) & 1)) * str;
        str *= nv_c;
      }
      for (int e = 0; e < dim; ++e) V[v * dim + e] = cv[idx * dim + e];
    }
    map_point(dim, V, xi, out);
  };
  m.n_cells = ipow(M, dim);
  const int nv = 1 << dim;
  m.vert.resize((size_t)m.n_cells * nv * dim);
  m.nbr.resize((size_t)m.n_cells * 2 * dim);
  m.speed.assign(m.n_cells, 1.0);
  m.density.assign(m.n_cells, 1.0);
  for (int64_t c = 0; c < m.n_cells; ++c) {
    int ic[3] = {0, 0, 0};
    int64_t t = c;
    for (int e = 0; e < dim; ++e) {
      ic[e] = (int)(t % M);
      t /= M;
    }
    for (int v = 0; v < nv; ++v) {
      int g[3];
      for (int e = 0; e < dim; ++e) g[e] = ic[e] + ((v >> e) & 1);
      fine_vertex(g, &m.vert[((size_t)c * nv + v) * dim]);
    }
    int64_t str = 1;
    for (int e = 0; e < dim; ++e) {
      m.nbr[c * 2 * dim + 2 * e] = ic[e] > 0 ? (int32_t)(c - str) : -bid;
      m.nbr[c * 2 * dim + 2 * e + 1] = ic[e] < M - 1 ? (int32_t)(c + str) : -bid;
      str *= M;
    }
  }
  return m;
}

// minimum distance between any two vertices of a cell
double min_vertex_distance(int dim, const double* V) {
  const int nv = 1 << dim;
  double best = 1e300;
  for (int a = 0; a < nv; ++a)
    for (int b = a + 1; b < nv; ++b) {
      double s = 0.0;
      for (int e = 0; e < dim; ++e) {
        const double d = V[a * dim + e] - V[b * dim + e];
        s += d * d;
      }
      best = std::min(best, std::sqrt(s));
    }
  return best;
}

// ---------------------------------------------------------------- operator
struct Oracle {
  int dim = 2, k = 1, n = 2, N = 4, F = 3;
  Mesh mesh;
  Basis1D B;
  std::vector<double> W;         // cell quadrature weights (tensor product)
  std::vector<char> cartesian;   // per cell: axis-aligned box
  std::vector<double> h;         // per cell extents (cartesian cells)
  int use_ader_post = 0;
  int spectral = 1;  // ADER: spectral evaluation with degree reduction (parameters.cc:76)
  // lower-degree collocation data for the ADER degree reduction
  std::vector<Basis1D> levels;     // levels[r]: n - 2r Gauss points
  std::vector<std::vector<double>> proj;    // proj[r]: (n_r-2) x n_r
  std::vector<std::vector<double>> interp;  // interp[r]: n_r x (n_r-2)
  std::string err;

  void setup() {
    n = k + 1;
    N = ipow(n, dim);
    F = dim + 1;
    B.init(n);
    W.assign(N, 1.0);
    for (int q = 0; q < N; ++q) {
      int t = q;
      for (int e = 0; e < dim; ++e) {
        W[q] *= B.rule.w[t % n];
        t /= n;
      }
    }
    const int nv = 1 << dim;
    cartesian.assign(mesh.n_cells, 0);
    h.assign(mesh.n_cells * dim, 0.0);
    for (int64_t c = 0; c < mesh.n_cells; ++c) {
      const double* V = &mesh.vert[(size_t)c * nv * dim];
      bool cart = true;
      for (int v = 0; v < nv && cart; ++v)
        for (int e = 0; e < dim; ++e) {
          const double ref = ((v >> e) & 1) ? V[(nv - 1) * dim + e] : V[e];
          if (V[v * dim + e] != ref) cart = false;
        }
      cartesian[c] = cart;
      for (int e = 0; e < dim; ++e) h[c * dim + e] = V[(nv - 1) * dim + e] - V[e];
    }
    // ADER levels: QGauss(k+1-2r), r = 0 .. k/2 (wave_equation_operations.cc:276-315)
    levels.clear();
    proj.clear();
    interp.clear();
    for (int r = 0; n - 2 * r >= 1; ++r) levels.emplace_back(n - 2 * r);
    for (size_t r = 0; r + 1 < levels.size(); ++r) {
      const Basis1D& hi = levels[r];
      const Basis1D& lo = levels[r + 1];
      std::vector<double> P(lo.n * hi.n), E(hi.n * lo.n);
      for (int i = 0; i < lo.n; ++i)
        for (int q = 0; q < hi.n; ++q) {
          const double v = lo.lag.value(i, hi.rule.x[q]);
          P[i * hi.n + q] = v * hi.rule.w[q] / lo.rule.w[i];
          E[q * lo.n + i] = v;
        }
      proj.push_back(P);
      interp.push_back(E);
    }
  }

  // geometry at a reference point: returns det J, fills JiT
  double geom(int64_t c, const double* xi, double JiT[3][3]) const {
    if (cartesian[c]) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) JiT[i][j] = 0.0;
      double det = 1.0;
      for (int e = 0; e < dim; ++e) {
        JiT[e][e] = 1.0 / h[c * dim + e];
        det *= h[c * dim + e];
      }
      return det;
    }
    double J[3][3];
    jacobian(dim, &mesh.vert[(size_t)c * (1 << dim) * dim], xi, J);
    return inverse_transpose(dim, J, JiT);
  }

  void point_index(int q, int* i) const {
    for (int e = 0; e < dim; ++e) {
      i[e] = q % n;
      q /= n;
    }
  }

  // dst = M^{-1} A(src) on one cell, scaled by bf (+1: RK operator,
  // -1: second ADER step).  Follows evaluate_cell (wave_equation_operations.cc:424-456),
  // evaluate_inner_face (480-551), evaluate_boundary_face (569-629) and the
  // inverse mass matrix (633-661); each cell evaluates its own side of every
  // face (the two sides of an interior face are mirror images of each other).
  void apply_cell(int64_t c, const double* src, double* dst, double bf,
                  std::vector<double>& R, std::vector<double>& G,
                  std::vector<double>& JxW) const {
    const int stride[3] = {1, n, n * n};
    const double* u = src + (size_t)c * F * N;
    const double rho = mesh.density[c], cc = mesh.speed[c];
    const double rho_inv = 1.0 / rho, c_sq = cc * cc;
    R.assign(F * N, 0.0);
    G.assign(dim * N, 0.0);
    JxW.assign(N, 0.0);
    // cell term
    for (int q = 0; q < N; ++q) {
      int i[3];
      point_index(q, i);
      double xi[3] = {0, 0, 0};
      for (int e = 0; e < dim; ++e) xi[e] = B.rule.x[i[e]];
      double JiT[3][3];
      const double det = geom(c, xi, JiT);
      JxW[q] = det * W[q];
      double gxi[3] = {0, 0, 0};
      for (int e = 0; e < dim; ++e)
        for (int a = 0; a < n; ++a)
          gxi[e] += B.D[i[e] * n + a] * u[dim * N + q + (a - i[e]) * stride[e]];
      for (int d = 0; d < dim; ++d) {
        double g = 0.0;
        for (int e = 0; e < dim; ++e) g += JiT[d][e] * gxi[e];
        R[d * N + q] += bf * (-rho_inv) * g * JxW[q];
      }
      for (int e = 0; e < dim; ++e) {
        double s = 0.0;
        for (int d = 0; d < dim; ++d) s += JiT[d][e] * u[d * N + q];
        G[e * N + q] = bf * rho * c_sq * JxW[q] * s;
      }
    }
    for (int q = 0; q < N; ++q) {
      int i[3];
      point_index(q, i);
      double s = 0.0;
      for (int e = 0; e < dim; ++e)
        for (int a = 0; a < n; ++a)
          s += B.D[a * n + i[e]] * G[e * N + q + (a - i[e]) * stride[e]];
      R[dim * N + q] += s;
    }
    // faces
    const int nf = ipow(n, dim - 1);
    for (int f = 0; f < 2 * dim; ++f) {
      const int e = f / 2, side = f % 2;
      const double* L = side ? B.L1.data() : B.L0.data();
      const double* Lm = side ? B.L0.data() : B.L1.data();
      const int nb = mesh.nbr[c * 2 * dim + f];
      int tdims[2], nt = 0;
      for (int d = 0; d < dim; ++d)
        if (d != e) tdims[nt++] = d;
      for (int t = 0; t < nf; ++t) {
        int ti[2] = {0, 0};
        {
          int tt = t;
          for (int a = 0; a < nt; ++a) {
            ti[a] = tt % n;
            tt /= n;
          }
        }
        int q0 = 0;
        double xi[3] = {0, 0, 0}, wt = 1.0;
        xi[e] = side ? 1.0 : 0.0;
        for (int a = 0; a < nt; ++a) {
          q0 += ti[a] * stride[tdims[a]];
          xi[tdims[a]] = B.rule.x[ti[a]];
          wt *= B.rule.w[ti[a]];
        }
        double JiT[3][3];
        const double det = geom(c, xi, JiT);
        double nrm[3] = {0, 0, 0}, len = 0.0;
        for (int d = 0; d < dim; ++d) {
          nrm[d] = (side ? 1.0 : -1.0) * JiT[d][e];
          len += nrm[d] * nrm[d];
        }
        len = std::sqrt(len);
        for (int d = 0; d < dim; ++d) nrm[d] /= len;
        const double jxw_f = wt * std::fabs(det) * len;
        double vp[4] = {0, 0, 0, 0};
        for (int fld = 0; fld < F; ++fld)
          for (int j = 0; j < n; ++j) vp[fld] += L[j] * u[fld * N + q0 + j * stride[e]];
        double un_p = 0.0;
        for (int d = 0; d < dim; ++d) un_p += vp[d] * nrm[d];
        double flux[4];
        if (nb >= 0) {
          const double* um = src + (size_t)nb * F * N;
          double vm[4] = {0, 0, 0, 0};
          for (int fld = 0; fld < F; ++fld)
            for (int j = 0; j < n; ++j) vm[fld] += Lm[j] * um[fld * N + q0 + j * stride[e]];
          double un_m = 0.0;
          for (int d = 0; d < dim; ++d) un_m -= vm[d] * nrm[d];
          const double rho_m = mesh.density[nb], c_m = mesh.speed[nb];
          const double tau_p = 1.0 / cc / rho, tau_m = 1.0 / c_m / rho_m;
          const double tau_inv = 1.0 / (tau_p + tau_m);
          const double lambda = tau_inv * (un_p + un_m + tau_p * vp[dim] + tau_m * vm[dim]);
          const double pd = (vp[dim] - lambda) * rho_inv;
          for (int d = 0; d < dim; ++d) flux[d] = bf * pd * nrm[d];
          flux[dim] = bf * c_sq * rho * (-un_p + tau_p * (lambda - vp[dim]));
        } else {
          const int id = -nb;
          const double tau = 1.0 / cc / rho;
          double lambda = 0.0;
          if (id == 1)
            lambda = 1.0 / tau * un_p + vp[dim];
          else if (id == 2)
            lambda = 0.0;
          else
            lambda = tau / (tau + 1.0 / cc / rho) * vp[dim] + 1.0 / (tau + 1.0 / cc / rho) * un_p;
          for (int d = 0; d < dim; ++d) flux[d] = bf * (vp[dim] - lambda) * rho_inv * nrm[d];
          flux[dim] = bf * c_sq * rho * (-un_p + tau * (lambda - vp[dim]));
        }
        for (int fld = 0; fld < F; ++fld) {
          const double fv = flux[fld] * jxw_f;
          for (int j = 0; j < n; ++j) R[fld * N + q0 + j * stride[e]] += L[j] * fv;
        }
      }
    }
    double* out = dst + (size_t)c * F * N;
    for (int fld = 0; fld < F; ++fld)
      for (int q = 0; q < N; ++q) out[fld * N + q] = R[fld * N + q] / JxW[q];
  }

  void apply(const double* src, double* dst, double bf = 1.0) const {
#pragma omp parallel
    {
      std::vector<double> R, G, JxW;
#pragma omp for schedule(static)
      for (int64_t c = 0; c < mesh.n_cells; ++c) apply_cell(c, src, dst, bf, R, G, JxW);
    }
  }

  size_t n_dofs() const { return (size_t)mesh.n_cells * F * N; }

  // ------------------------------------------------------------ ADER CK
  // Physical gradient-type derivative at level r of a field set S (F fields
  // at n_r^dim points): out_u_d = rho^{-1} d_d S_p, out_p = rho c^2 div S_u.
  void ck_derivative(int64_t c, int r, const std::vector<double>& S,
                     std::vector<double>& out, double rho, double c_sq) const {
    const Basis1D& b = levels[r];
    const int m = b.n, Nm = ipow(m, dim);
    const int stride[3] = {1, m, m * m};
    out.assign(F * Nm, 0.0);
    const double rho_inv = 1.0 / rho;
    for (int q = 0; q < Nm; ++q) {
      int i[3] = {0, 0, 0};
      {
        int t = q;
        for (int e = 0; e < dim; ++e) {
          i[e] = t % m;
          t /= m;
        }
      }
      double xi[3] = {0, 0, 0};
      for (int e = 0; e < dim; ++e) xi[e] = b.rule.x[i[e]];
      double JiT[3][3];
      geom(c, xi, JiT);
      // reference gradients of all fields
      double g[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int fld = 0; fld < F; ++fld)
        for (int e = 0; e < dim; ++e) {
          double s = 0.0;
          for (int a = 0; a < m; ++a) s += b.D[i[e] * m + a] * S[fld * Nm + q + (a - i[e]) * stride[e]];
          g[fld][e] = s;
        }
      double div = 0.0;
      for (int d = 0; d < dim; ++d)
        for (int e = 0; e < dim; ++e) div += g[d][e] * JiT[d][e];
      for (int d = 0; d < dim; ++d) {
        double pg = 0.0;
        for (int e = 0; e < dim; ++e) pg += g[dim][e] * JiT[d][e];
        out[d * Nm + q] = rho_inv * pg;
      }
      out[dim * Nm + q] = c_sq * rho * div;
    }
  }

  // tensor-product application of a 1D matrix A (rows x cols) in every
  // direction to F fields: in has cols^dim points, out rows^dim points
  void tensor_apply(const std::vector<double>& A, int rows, int cols,
                    const std::vector<double>& in, std::vector<double>& out) const {
    const int Nin = ipow(cols, dim), Nout = ipow(rows, dim);
    out.assign(F * Nout, 0.0);
    std::vector<double> cur, nxt;
    for (int fld = 0; fld < F; ++fld) {
      cur.assign(in.begin() + fld * Nin, in.begin() + (fld + 1) * Nin);
      int ext[3] = {cols, cols, cols};
      for (int e = 0; e < dim; ++e) {
        int newext[3] = {ext[0], ext[1], ext[2]};
        newext[e] = rows;
        int tot = 1;
        for (int a = 0; a < dim; ++a) tot *= newext[a];
        nxt.assign(tot, 0.0);
        for (int idx = 0; idx < tot; ++idx) {
          int ii[3] = {0, 0, 0}, t = idx;
          for (int a = 0; a < dim; ++a) {
            ii[a] = t % newext[a];
            t /= newext[a];
          }
          double s = 0.0;
          for (int j = 0; j < cols; ++j) {
            int jj[3] = {ii[0], ii[1], ii[2]};
            jj[e] = j;
            int src = 0, str = 1;
            for (int a = 0; a < dim; ++a) {
              src += jj[a] * str;
              str *= ext[a];
            }
            s += A[ii[e] * cols + j] * cur[src];
          }
          nxt[idx] = s;
        }
        cur.swap(nxt);
        ext[e] = rows;
      }
      std::copy(cur.begin(), cur.end(), out.begin() + fld * Nout);
    }
  }

  // Time integral T = int_0^dt u dt of one cell via the Taylor /
  // Cauchy-Kovalevskaya procedure with spectral evaluation and degree
  // reduction every second derivative (integrate_taylor_cauchykovalewski,
  // wave_equation_operations.cc:961-1059, and its recursive step 1063-1262).
  // Without spectral evaluation (:1013, 1037, 1086-1090, 1205-1233) every
  // derivative is submitted, integrated, multiplied by the inverse mass
  // matrix and its gradient evaluated at the full degree: in the Gauss
  // collocation basis the first three are the identity, so the recursion runs
  // on level 0 throughout and no degree is reduced.
  // `d1` holds the values of the first time derivative when use_ader_post
  // is set (the full DG operator applied to src), else null.
  void ck_cell(int64_t c, const double* src, const double* d1, double dt, double* T) const {
    const double rho = mesh.density[c], cc = mesh.speed[c];
    const double rho_inv = 1.0 / rho, c_sq = cc * cc;
    const double* u = src + (size_t)c * F * N;
    const int nlev = (int)levels.size();
    std::vector<std::vector<double>> contrib(nlev);
    contrib[0].assign(F * N, 0.0);
    std::vector<double> S(F * N), D1(F * N);
    for (int i = 0; i < F * N; ++i) contrib[0][i] = dt * u[i];
    if (d1) {
      for (int i = 0; i < F * N; ++i) D1[i] = d1[(size_t)c * F * N + i];
    } else {
      // cell-local first derivative: (-rho^{-1} grad p, -rho c^2 div u)
      std::vector<double> Uv(u, u + F * N), tmp;
      ck_derivative(c, 0, Uv, tmp, rho, c_sq);
      for (int i = 0; i < F * N; ++i) D1[i] = -tmp[i];
      (void)rho_inv;
    }
    for (int i = 0; i < F * N; ++i) {
      contrib[0][i] += dt * dt * 0.5 * D1[i];
      S[i] = -D1[i];
    }
    const int n_steps = std::max(1, k - 1);
    int r = 0;
    std::vector<double> Snew, Sproj;
    for (int s = 0; s < n_steps; ++s) {
      r = spectral ? s / 2 : 0;
      if (contrib[r].empty()) contrib[r].assign(F * ipow(levels[r].n, dim), 0.0);
      ck_derivative(c, r, S, Snew, rho, c_sq);
      double fac = -0.5;
      for (int kk = 2; kk <= s + 2; ++kk) fac /= -(kk + 1.0);
      const double fac_t = fac * std::pow(dt, s + 3);
      for (size_t i = 0; i < Snew.size(); ++i) contrib[r][i] += fac_t * Snew[i];
      S.swap(Snew);
      if (spectral && s + 1 < n_steps && (s % 2) == 1) {
        tensor_apply(proj[r], levels[r + 1].n, levels[r].n, S, Sproj);
        S.swap(Sproj);
      }
    }
    for (int rr = nlev - 1; rr >= 1; --rr) {
      if (contrib[rr].empty()) continue;
      std::vector<double> up;
      tensor_apply(interp[rr - 1], levels[rr - 1].n, levels[rr].n, contrib[rr], up);
      for (size_t i = 0; i < up.size(); ++i) contrib[rr - 1][i] += up[i];
    }
    std::copy(contrib[0].begin(), contrib[0].end(), T + (size_t)c * F * N);
  }
};

// ---------------------------------------------------------------- errors
struct ModeSet {
  // p = sum_m A_m cos(w_m t) prod_d sin(k_{m,d} pi x_d) (c = rho = 1)
  std::vector<double> amp;
  std::vector<int> kv;  // [mode][3]
};

void exact_membrane(int dim, const ModeSet& ms, const double* x, double t, double* out) {
  for (int f = 0; f <= dim; ++f) out[f] = 0.0;
  for (size_t m = 0; m < ms.amp.size(); ++m) {
    double ksq = 0.0;
    for (int d = 0; d < dim; ++d) ksq += (double)ms.kv[m * 3 + d] * ms.kv[m * 3 + d];
    const double w = kPi * std::sqrt(ksq);
    double prod = 1.0;
    for (int d = 0; d < dim; ++d) prod *= std::sin(ms.kv[m * 3 + d] * kPi * x[d]);
    out[dim] += ms.amp[m] * std::cos(w * t) * prod;
    for (int c = 0; c < dim; ++c) {
      double v = -ms.amp[m] * (ms.kv[m * 3 + c] * kPi / w) * std::sin(w * t);
      for (int d = 0; d < dim; ++d)
        v *= (d == c) ? std::cos(ms.kv[m * 3 + d] * kPi * x[d]) : std::sin(ms.kv[m * 3 + d] * kPi * x[d]);
      out[c] += v;
    }
  }
}

// The reference's single-mode solution (input_parameters.h:95-128): mode m in
// every direction, omega = m sqrt(dim) pi.  Evaluated with the reference's
// own formula, not through ModeSet, so both the printed errors and the
// generalisation are pinned.
void exact_reference(int dim, int m, const double* x, double t, double* out) {
  const double w = m * std::sqrt((double)dim) * kPi;
  for (int comp = 0; comp <= dim; ++comp) {
    double v = (comp == dim) ? std::cos(w * t) : -std::sin(w * t) / std::sqrt((double)dim);
    for (int d = 0; d < dim; ++d)
      v *= (d != comp) ? std::sin(m * kPi * x[d]) : std::cos(m * kPi * x[d]);
    out[comp] = v;
  }
}

// L2 errors with QGauss(k+2) on the mapped cells (explicit_wave.cc:439-496):
// out[0] = ||p_h - p||, out[1] = ||u_h - u||, out[2] = ||p||.
template <class Exact>
void l2_errors(const Oracle& O, const double* sol, Exact exact, double* out) {
  const int dim = O.dim, n = O.n, F = O.F, N = O.N;
  const Rule qr = gauss_rule(n + 1);
  const int m = qr.n, M = ipow(m, dim);
  std::vector<double> I(m * n);
  for (int a = 0; a < m; ++a)
    for (int i = 0; i < n; ++i) I[a * n + i] = O.B.lag.value(i, qr.x[a]);
  std::vector<double> Iv(I);
  double ep = 0.0, ev = 0.0, mag = 0.0;
#pragma omp parallel reduction(+ : ep, ev, mag)
  {
    std::vector<double> vals;
    std::vector<double> cellv;
#pragma omp for schedule(static)
    for (int64_t c = 0; c < O.mesh.n_cells; ++c) {
      cellv.assign(sol + (size_t)c * F * N, sol + (size_t)(c + 1) * F * N);
      O.tensor_apply(Iv, m, n, cellv, vals);
      const double* V = &O.mesh.vert[(size_t)c * (1 << dim) * dim];
      for (int qp = 0; qp < M; ++qp) {
        int ii[3] = {0, 0, 0}, t = qp;
        double xi[3] = {0, 0, 0}, w = 1.0;
        for (int e = 0; e < dim; ++e) {
          ii[e] = t % m;
          t /= m;
          xi[e] = qr.x[ii[e]];
          w *= qr.w[ii[e]];
        }
        double J[3][3], JiT[3][3], x[3] = {0, 0, 0};
        jacobian(dim, V, xi, J);
        const double det = inverse_transpose(dim, J, JiT);
        map_point(dim, V, xi, x);
        const double jxw = std::fabs(det) * w;
        double ex[4];
        exact(x, ex);
        const double dp = vals[dim * M + qp] - ex[dim];
        ep += dp * dp * jxw;
        mag += ex[dim] * ex[dim] * jxw;
        for (int d = 0; d < dim; ++d) {
          const double dv = vals[d * M + qp] - ex[d];
          ev += dv * dv * jxw;
        }
      }
    }
  }
  out[0] = std::sqrt(ep);
  out[1] = std::sqrt(ev);
  out[2] = std::sqrt(mag);
}

// WaveEquationOperation::compute_post_pressure (wave_equation_operations.cc:784-848)
// and the "error p post" of output_results (explicit_wave.cc:476-484): on
// every cell the Q_{k+1} pressure p* with (grad phi, grad p*) =
// (grad phi, -rho du/dt) for all phi in Q_{k+1} (QGauss(k+2) on the mapped
// cell; du/dt is the velocity part of M^-1 A(u)), solved with the
// reference's unpreconditioned CG (first unknown constrained, relative
// tolerance 1e-11), shifted to the mean of p, and its L2 error against the
// exact pressure with QGauss(k+3).  p* is written by its values at the
// QGauss(k+2) points (any basis of Q_{k+1} gives the same function).
template <class Exact>
double post_pressure_error(Oracle& O, const double* sol, Exact exact) {
  const int dim = O.dim, n = O.n, F = O.F, N = O.N;
  std::vector<double> tmp((size_t)O.n_dofs());
  O.apply(sol, tmp.data());
  const int m = n + 1, Mp = ipow(m, dim);
  Basis1D P(m);                    // Lagrange basis at the QGauss(k+2) points
  std::vector<double> I(m * n);    // Q_k values at n Gauss points -> m points
  for (int a = 0; a < m; ++a)
    for (int i = 0; i < n; ++i) I[a * n + i] = O.B.lag.value(i, P.rule.x[a]);
  const Rule er = gauss_rule(m + 1);  // QGauss(k+3)
  const int me = er.n, Me = ipow(me, dim);
  std::vector<double> Ie(me * m);
  for (int a = 0; a < me; ++a)
    for (int i = 0; i < m; ++i) Ie[a * m + i] = P.lag.value(i, er.x[a]);
  const double ABS_TOL = 1e-20, REL_TOL = 1e-11;
  double esum = 0.0;
#pragma omp parallel reduction(+ : esum)
  {
    std::vector<double> cellv, vq, pq, jxw(Mp), met(Mp * 9), rhs(Mp), x(Mp), r(Mp), pv(Mp), v(Mp),
        g(3 * Mp), xe;
    // y = K x: the Laplacian (grad phi_i, grad phi_j) with unknown 0 constrained
    auto lap = [&](const std::vector<double>& in, std::vector<double>& out) {
      std::vector<double> z(in);
      z[0] = 0.0;
      for (int q = 0; q < Mp; ++q) {
        int ii[3] = {0, 0, 0}, t = q, str[3] = {1, m, m * m};
        for (int e = 0; e < dim; ++e) {
          ii[e] = t % m;
          t /= m;
        }
        double gr[3] = {0, 0, 0};
        for (int e = 0; e < dim; ++e)
          for (int a = 0; a < m; ++a) gr[e] += P.D[ii[e] * m + a] * z[q + (a - ii[e]) * str[e]];
        for (int e = 0; e < dim; ++e) {
          double s = 0.0;
          for (int f = 0; f < dim; ++f) s += met[q * 9 + e * 3 + f] * gr[f];
          g[e * Mp + q] = jxw[q] * s;
        }
      }
      for (int i = 0; i < Mp; ++i) {
        int ii[3] = {0, 0, 0}, t = i, str[3] = {1, m, m * m};
        for (int e = 0; e < dim; ++e) {
          ii[e] = t % m;
          t /= m;
        }
        double s = 0.0;
        for (int e = 0; e < dim; ++e)
          for (int a = 0; a < m; ++a) s += P.D[a * m + ii[e]] * g[e * Mp + i + (a - ii[e]) * str[e]];
        out[i] = s;
      }
      out[0] = in[0];
    };
    auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
      double s = 0.0;
      for (int i = 0; i < Mp; ++i) s += a[i] * b[i];
      return s;
    };
#pragma omp for schedule(dynamic, 4)
    for (int64_t c = 0; c < O.mesh.n_cells; ++c) {
      const double* V = &O.mesh.vert[(size_t)c * (1 << dim) * dim];
      const double rho = O.mesh.density[c];
      cellv.assign(tmp.begin() + (size_t)c * F * N, tmp.begin() + (size_t)(c + 1) * F * N);
      O.tensor_apply(I, m, n, cellv, vq);  // du/dt at the m^dim points (fields 0..dim-1)
      cellv.assign(sol + (size_t)c * F * N, sol + (size_t)(c + 1) * F * N);
      O.tensor_apply(I, m, n, cellv, pq);  // p at the m^dim points (field dim)
      double vol = 0.0, pint = 0.0;
      for (int q = 0; q < Mp; ++q) {
        int t = q;
        double xi[3] = {0, 0, 0}, w = 1.0;
        for (int e = 0; e < dim; ++e) {
          xi[e] = P.rule.x[t % m];
          w *= P.rule.w[t % m];
          t /= m;
        }
        double J[3][3], JiT[3][3];
        jacobian(dim, V, xi, J);
        jxw[q] = std::fabs(inverse_transpose(dim, J, JiT)) * w;
        for (int e = 0; e < dim; ++e)
          for (int f = 0; f < dim; ++f) {
            double s = 0.0;
            for (int d = 0; d < dim; ++d) s += JiT[d][e] * JiT[d][f];
            met[q * 9 + e * 3 + f] = s;
          }
        // reference-coordinate flux of -rho du/dt: sum_d JiT[d][e] (-rho v_d)
        for (int e = 0; e < dim; ++e) {
          double s = 0.0;
          for (int d = 0; d < dim; ++d) s += JiT[d][e] * (-rho * vq[d * Mp + q]);
          g[e * Mp + q] = jxw[q] * s;
        }
        vol += jxw[q];
        pint += jxw[q] * pq[dim * Mp + q];
      }
      for (int i = 0; i < Mp; ++i) {
        int ii[3] = {0, 0, 0}, t = i, str[3] = {1, m, m * m};
        for (int e = 0; e < dim; ++e) {
          ii[e] = t % m;
          t /= m;
        }
        double s = 0.0;
        for (int e = 0; e < dim; ++e)
          for (int a = 0; a < m; ++a) s += P.D[a * m + ii[e]] * g[e * Mp + i + (a - ii[e]) * str[e]];
        rhs[i] = s;
      }
      rhs[0] = 0.0;
      // SolverCGvect::solve (elementwise_cg.templates.h:64-145), identity preconditioner
      std::fill(x.begin(), x.end(), 0.0);
      r = rhs;
      const double r0 = std::sqrt(dot(r, r));
      if (r0 > 0.0) {
        pv = r;
        double ry = dot(r, pv);
        for (int it = 1; it <= 6 * Mp; ++it) {
          lap(pv, v);
          double pvv = dot(pv, v);
          if (std::fabs(pvv) < ABS_TOL) pvv = ABS_TOL;
          const double alpha = ry / pvv;
          for (int i = 0; i < Mp; ++i) {
            x[i] += alpha * pv[i];
            r[i] -= alpha * v[i];
          }
          const double rn = std::sqrt(dot(r, r));
          if (rn < ABS_TOL || rn / r0 < REL_TOL) break;
          const double ry_new = dot(r, r);
          const double beta = ry_new / ry;
          for (int i = 0; i < Mp; ++i) pv[i] = r[i] + beta * pv[i];
          ry = ry_new;
        }
      }
      // mean of p
      double sint = 0.0;
      for (int q = 0; q < Mp; ++q) sint += jxw[q] * x[q];
      const double shift = (pint - sint) / vol;
      for (int q = 0; q < Mp; ++q) x[q] += shift;
      // error with QGauss(k+3)
      xe.assign(Me, 0.0);
      {
        // tensor interpolation of the single field x from m to me points
        std::vector<double> cur(x), nxt;
        int ext[3] = {m, m, m};
        for (int e = 0; e < dim; ++e) {
          int sz_out = 1;
          for (int f = 0; f < dim; ++f) sz_out *= (f == e ? me : ext[f]);
          nxt.assign(sz_out, 0.0);
          const int s0 = (e == 0) ? 1 : (e == 1 ? ext[0] : ext[0] * ext[1]);
          for (int o = 0; o < sz_out; ++o) {
            int idx[3] = {0, 0, 0}, t = o;
            for (int f = 0; f < dim; ++f) {
              const int ef = (f == e) ? me : ext[f];
              idx[f] = t % ef;
              t /= ef;
            }
            int base = 0, mul = 1;
            for (int f = 0; f < dim; ++f) {
              base += (f == e ? 0 : idx[f]) * mul;
              mul *= ext[f];
            }
            double s = 0.0;
            for (int a = 0; a < m; ++a) s += Ie[idx[e] * m + a] * cur[base + a * s0];
            nxt[o] = s;
          }
          cur.swap(nxt);
          ext[e] = me;
        }
        xe = cur;
      }
      for (int q = 0; q < Me; ++q) {
        int t = q;
        double xi[3] = {0, 0, 0}, w = 1.0;
        for (int e = 0; e < dim; ++e) {
          xi[e] = er.x[t % me];
          w *= er.w[t % me];
          t /= me;
        }
        double J[3][3], JiT[3][3], xp[3] = {0, 0, 0}, ex[4];
        jacobian(dim, V, xi, J);
        const double jw = std::fabs(inverse_transpose(dim, J, JiT)) * w;
        map_point(dim, V, xi, xp);
        exact(xp, ex);
        const double d = xe[q] - ex[dim];
        esum += d * d * jw;
      }
    }
  }
  return std::sqrt(esum);
}

thread_local std::string g_last_error;

}  // namespace

// ============================================================= C interface
extern "C" {

struct ewo_problem;

const char* ewo_last_error() { return g_last_error.c_str(); }

// Build an oracle over an explicit mesh (same arrays as ew_mesh_desc).
ewo_problem* ewo_create(int dim, int degree, int64_t n_cells, const double* vertices,
                        const int32_t* neighbors, const double* speed, const double* density) {
  if ((dim != 2 && dim != 3) || degree < 1 || degree > 12 || n_cells <= 0) {
    g_last_error = "ewo_create: invalid dim/degree/n_cells";
    return nullptr;
  }
  Oracle* O = new Oracle;
  O->dim = dim;
  O->k = degree;
  O->mesh.dim = dim;
  O->mesh.n_cells = n_cells;
  const int nv = 1 << dim;
  O->mesh.vert.assign(vertices, vertices + (size_t)n_cells * nv * dim);
  O->mesh.nbr.assign(neighbors, neighbors + (size_t)n_cells * 2 * dim);
  O->mesh.speed.assign(speed, speed + n_cells);
  O->mesh.density.assign(density, density + n_cells);
  O->setup();
  return reinterpret_cast<ewo_problem*>(O);
}

// The reference's mesh for a parameter set (make_grid, explicit_wave.cc:177-195).
ewo_problem* ewo_create_hypercube(int dim, int degree, int n_intervals, int n_refinements,
                                  double transform_factor, int boundary_id) {
  Mesh m = hypercube_mesh(dim, n_intervals, n_refinements, transform_factor, boundary_id);
  return ewo_create(dim, degree, m.n_cells, m.vert.data(), m.nbr.data(), m.speed.data(),
                    m.density.data());
}

void ewo_destroy(ewo_problem* p) { delete reinterpret_cast<Oracle*>(p); }

int64_t ewo_n_cells(ewo_problem* p) { return reinterpret_cast<Oracle*>(p)->mesh.n_cells; }
int64_t ewo_n_dofs(ewo_problem* p) { return (int64_t) reinterpret_cast<Oracle*>(p)->n_dofs(); }
const double* ewo_vertices(ewo_problem* p) { return reinterpret_cast<Oracle*>(p)->mesh.vert.data(); }
const int32_t* ewo_neighbors(ewo_problem* p) { return reinterpret_cast<Oracle*>(p)->mesh.nbr.data(); }
void ewo_set_ader_post(ewo_problem* p, int on) { reinterpret_cast<Oracle*>(p)->use_ader_post = on; }
void ewo_set_spectral(ewo_problem* p, int on) { reinterpret_cast<Oracle*>(p)->spectral = on; }

// dt = cfl * min_cells(min vertex distance / c) (explicit_wave.cc:529-545);
// cfl is the already-scaled Courant number (parameters.cc:195).
double ewo_time_step(ewo_problem* p, double cfl) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  double best = 1e300;
  const int nv = 1 << O->dim;
  for (int64_t c = 0; c < O->mesh.n_cells; ++c)
    best = std::min(best, min_vertex_distance(O->dim, &O->mesh.vert[(size_t)c * nv * O->dim]) /
                              O->mesh.speed[c]);
  return cfl * best;
}

// physical coordinates of all Gauss points: [cell][point][dim]
void ewo_quadrature_points(ewo_problem* p, double* xyz) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int nv = 1 << O->dim;
  for (int64_t c = 0; c < O->mesh.n_cells; ++c)
    for (int q = 0; q < O->N; ++q) {
      int i[3] = {0, 0, 0};
      O->point_index(q, i);
      double xi[3] = {0, 0, 0};
      for (int e = 0; e < O->dim; ++e) xi[e] = O->B.rule.x[i[e]];
      map_point(O->dim, &O->mesh.vert[(size_t)c * nv * O->dim], xi,
                xyz + ((size_t)c * O->N + q) * O->dim);
    }
}

// Initial field of the reference (single membrane mode m, t = 0).
void ewo_project_reference(ewo_problem* p, int modes, double t, double* u) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  std::vector<double> xyz((size_t)O->mesh.n_cells * O->N * O->dim);
  ewo_quadrature_points(p, xyz.data());
  for (int64_t c = 0; c < O->mesh.n_cells; ++c)
    for (int q = 0; q < O->N; ++q) {
      double ex[4];
      exact_reference(O->dim, modes, &xyz[((size_t)c * O->N + q) * O->dim], t, ex);
      for (int f = 0; f < O->F; ++f) u[(size_t)c * O->F * O->N + f * O->N + q] = ex[f];
    }
}

// Multi-mode membrane field (amplitudes amp[m], integer wave numbers kv[m][3]).
void ewo_project_modes(ewo_problem* p, int n_modes, const double* amp, const int* kv, double t,
                       double* u) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  ModeSet ms;
  ms.amp.assign(amp, amp + n_modes);
  ms.kv.assign(kv, kv + 3 * n_modes);
  std::vector<double> xyz((size_t)O->mesh.n_cells * O->N * O->dim);
  ewo_quadrature_points(p, xyz.data());
  for (int64_t c = 0; c < O->mesh.n_cells; ++c)
    for (int q = 0; q < O->N; ++q) {
      double ex[4];
      exact_membrane(O->dim, ms, &xyz[((size_t)c * O->N + q) * O->dim], t, ex);
      for (int f = 0; f < O->F; ++f) u[(size_t)c * O->F * O->N + f * O->N + q] = ex[f];
    }
}

// Gaussian pressure pulse p = amp exp(-|x - x0|^2 / (2 width^2)), u = 0,
// sampled at the Gauss points (the L2 projection in the collocation basis,
// project_initial_field, wave_equation_operations.cc:902-935).  The pulse
// itself has no counterpart in the reference; it is the initial field of
// the curved two-layer ADER configuration.
void ewo_project_gaussian(ewo_problem* p, const double* x0, double width, double amp, double* u) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  std::vector<double> xyz((size_t)O->mesh.n_cells * O->N * O->dim);
  ewo_quadrature_points(p, xyz.data());
  for (int64_t c = 0; c < O->mesh.n_cells; ++c)
    for (int q = 0; q < O->N; ++q) {
      const double* x = &xyz[((size_t)c * O->N + q) * O->dim];
      double r2 = 0.0;
      for (int e = 0; e < O->dim; ++e) r2 += (x[e] - x0[e]) * (x[e] - x0[e]);
      for (int f = 0; f < O->dim; ++f) u[(size_t)c * O->F * O->N + f * O->N + q] = 0.0;
      u[(size_t)c * O->F * O->N + O->dim * O->N + q] = amp * std::exp(-r2 / (2.0 * width * width));
    }
}

void ewo_apply(ewo_problem* p, const double* src, double* dst, double boundary_fac) {
  reinterpret_cast<Oracle*>(p)->apply(src, dst, boundary_fac);
}

// RKVectorUpdater (time_integrators.cc:129-155)
void ewo_rk_update(int64_t n, double f1, double f2, int is_last, const double* v1, double* v2,
                   double* v3) {
  if (is_last) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) v2[i] = v3[i] + f1 * v1[i];
  } else {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const double up = v1[i];
      v2[i] += f1 * up;
      v3[i] = v2[i] + f2 * up;
    }
  }
}

// LowStorageRK45Reg2::perform_time_step (time_integrators.cc:235-283):
// vec_n is clobbered, the new state is written to vec_np.
void ewo_lsrk45_step(ewo_problem* p, double dt, double* vec_n, double* vec_np) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int64_t nd = (int64_t)O->n_dofs();
  std::vector<double> tmp(nd);
  const double a21 = 970286171893. / 4311952581923.;
  const double a32 = 6584761158862. / 12103376702013.;
  const double a43 = 2251764453980. / 15575788980749.;
  const double a54 = 26877169314380. / 34165994151039.;
  const double b1 = 1153189308089. / 22510343858157.;
  const double b2 = 1772645290293. / 4653164025191.;
  const double b3 = -1672844663538. / 4480602732383.;
  const double b4 = 2114624349019. / 3568978502595.;
  const double b5 = 5198255086312. / 14908931495163.;
  O->apply(vec_n, tmp.data());
  ewo_rk_update(nd, a21 * dt, (b1 - a21) * dt, 0, tmp.data(), vec_n, vec_np);
  O->apply(vec_n, tmp.data());
  ewo_rk_update(nd, a32 * dt, (b2 - a32) * dt, 0, tmp.data(), vec_np, vec_n);
  O->apply(vec_np, tmp.data());
  ewo_rk_update(nd, a43 * dt, (b3 - a43) * dt, 0, tmp.data(), vec_n, vec_np);
  O->apply(vec_n, tmp.data());
  ewo_rk_update(nd, a54 * dt, (b4 - a54) * dt, 0, tmp.data(), vec_np, vec_n);
  O->apply(vec_np, tmp.data());
  ewo_rk_update(nd, b5 * dt, 0.0, 1, tmp.data(), vec_np, vec_n);
}

// ClassRK4::perform_time_step (time_integrators.cc:66-102)
void ewo_clrk4_step(ewo_problem* p, double dt, double* vec_n, double* vec_np) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int64_t nd = (int64_t)O->n_dofs();
  std::vector<double> t1(nd), t2(nd);
  O->apply(vec_n, t1.data());
  for (int64_t i = 0; i < nd; ++i) {
    vec_np[i] = vec_n[i] + dt / 6. * t1[i];
    t2[i] = vec_n[i] + 0.5 * dt * t1[i];
  }
  O->apply(t2.data(), t1.data());
  for (int64_t i = 0; i < nd; ++i) {
    vec_np[i] += dt / 3. * t1[i];
    t2[i] = vec_n[i] + 0.5 * dt * t1[i];
  }
  O->apply(t2.data(), t1.data());
  for (int64_t i = 0; i < nd; ++i) {
    vec_np[i] += dt / 3. * t1[i];
    t2[i] = vec_n[i] + dt * t1[i];
  }
  O->apply(t2.data(), t1.data());
  for (int64_t i = 0; i < nd; ++i) vec_np[i] += dt / 6. * t1[i];
}

// ExplicitEuler::perform_time_step (time_integrators.cc:24-31):
// vec_np = M^-1 A(vec_n), then vec_np = dt vec_np + vec_n (Vector::sadd).
void ewo_expleuler_step(ewo_problem* p, double dt, double* vec_n, double* vec_np) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int64_t nd = (int64_t)O->n_dofs();
  O->apply(vec_n, vec_np);
  for (int64_t i = 0; i < nd; ++i) vec_np[i] = dt * vec_np[i] + vec_n[i];
}

// Low-storage 2-register schemes in the form of LowStorageRK33Reg2 /
// LowStorageRK45Reg2 / LowStorageRK59Reg2 (time_integrators.cc:200-364):
// stage s applies the operator to the current stage input and calls the
// RKVectorUpdater with (a_{s+1,s} dt, (b_s - a_{s+1,s}) dt); the roles of
// vec_n and vec_np alternate, the last stage adds b_n dt.  a[n-1], b[n].
static void lsrk2r_step(Oracle* O, int n, const double* a, const double* b, double dt,
                        double* vec_n, double* vec_np) {
  const int64_t nd = (int64_t)O->n_dofs();
  std::vector<double> tmp(nd);
  for (int s = 0; s < n; ++s) {
    // stage input: vec_n in the first stage, then the vector the previous
    // update wrote as its second argument (vec_n after even, vec_np after
    // odd stages)
    const double* in = (s == 0 || (s & 1)) ? vec_n : vec_np;
    O->apply(in, tmp.data());
    if (s + 1 == n)
      ewo_rk_update(nd, b[s] * dt, 0.0, 1, tmp.data(), vec_np, vec_n);
    else if (s & 1)
      ewo_rk_update(nd, a[s] * dt, (b[s] - a[s]) * dt, 0, tmp.data(), vec_np, vec_n);
    else
      ewo_rk_update(nd, a[s] * dt, (b[s] - a[s]) * dt, 0, tmp.data(), vec_n, vec_np);
  }
}

// LowStorageRK33Reg2 coefficients (time_integrators.cc:206-211)
void ewo_lsrk33_step(ewo_problem* p, double dt, double* vec_n, double* vec_np) {
  const double a[2] = {0.755726351946097, 0.386954477304099};
  const double b[3] = {0.245170287303492, 0.184896052186740, 0.569933660509768};
  lsrk2r_step(reinterpret_cast<Oracle*>(p), 3, a, b, dt, vec_n, vec_np);
}

// LowStorageRK59Reg2 coefficients (time_integrators.cc:294-311)
void ewo_lsrk59_step(ewo_problem* p, double dt, double* vec_n, double* vec_np) {
  const double a[8] = {1107026461565. / 5417078080134.,   38141181049399. / 41724347789894.,
                       493273079041. / 11940823631197.,   1851571280403. / 6147804934346.,
                       11782306865191. / 62590030070788., 9452544825720. / 13648368537481.,
                       4435885630781. / 26285702406235.,  2357909744247. / 11371140753790.};
  const double b[9] = {2274579626619. / 23610510767302.,  693987741272. / 12394497460941.,
                       -347131529483. / 15096185902911.,  1144057200723. / 32081666971178.,
                       1562491064753. / 11797114684756.,  13113619727965. / 44346030145118.,
                       393957816125. / 7825732611452.,    720647959663. / 6565743875477.,
                       3559252274877. / 14424734981077.};
  lsrk2r_step(reinterpret_cast<Oracle*>(p), 9, a, b, dt, vec_n, vec_np);
}

// y = alpha y + (beta x + gamma z): Vector::add(a, V, b, W) (alpha = 1),
// Vector::sadd(s, a, V) (gamma = 0) and assignment (alpha = 0, beta = 1)
static void vec_update(int64_t n, double alpha, double* y, double beta, const double* x,
                       double gamma, const double* z) {
  for (int64_t i = 0; i < n; ++i) {
    const double xz = (x ? beta * x[i] : 0.0) + (z ? gamma * z[i] : 0.0);
    y[i] = alpha == 0.0 ? xz : alpha * y[i] + xz;
  }
}

// LowStorageRK45Reg3::perform_time_step (time_integrators.cc:366-427),
// the same sequence of operator applications and vector operations.
void ewo_lsrk45r3_step(ewo_problem* p, double dt, double* vec_n, double* vec_np) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int64_t nd = (int64_t)O->n_dofs();
  const double a21 = 2365592473904. / 8146167614645., a32 = 4278267785271. / 6823155464066.,
               a43 = 2789585899612. / 8986505720531., a54 = 15310836689591. / 24358012670437.;
  const double a31 = -722262345248. / 10870640012513., a42 = 1365858020701. / 8494387045469.,
               a53 = 3819021186. / 2763618202291.;
  const double b1 = 846876320697. / 6523801458457., b2 = 3032295699695. / 12397907741132.,
               b3 = 612618101729. / 6534652265123., b4 = 1155491934595. / 2954287928812.,
               b5 = 707644755468. / 5028292464395.;
  std::vector<double> t1(nd), t2(nd);
  O->apply(vec_n, vec_np);
  vec_update(nd, 1.0, vec_n, a21 * dt, vec_np, 0.0, nullptr);
  vec_update(nd, 0.0, t1.data(), 1.0, vec_n, 0.0, nullptr);
  vec_update(nd, 1.0, t1.data(), (b1 - a21) * dt, vec_np, 0.0, nullptr);
  O->apply(vec_n, t2.data());
  vec_update(nd, 1.0, t1.data(), a32 * dt, t2.data(), (a31 - b1) * dt, vec_np);
  vec_update(nd, (b1 - a31) * dt, vec_np, 1.0, t1.data(), 0.0, nullptr);
  vec_update(nd, 1.0, vec_np, (b2 - a32) * dt, t2.data(), 0.0, nullptr);
  O->apply(t1.data(), vec_n);
  vec_update(nd, 1.0, vec_np, a43 * dt, vec_n, (a42 - b2) * dt, t2.data());
  vec_update(nd, (b2 - a42) * dt, t2.data(), 1.0, vec_np, 0.0, nullptr);
  vec_update(nd, 1.0, t2.data(), (b3 - a43) * dt, vec_n, 0.0, nullptr);
  O->apply(vec_np, t1.data());
  vec_update(nd, 1.0, t2.data(), a54 * dt, t1.data(), (a53 - b3) * dt, vec_n);
  vec_update(nd, 0.0, vec_np, 1.0, t2.data(), 0.0, nullptr);
  vec_update(nd, 1.0, vec_np, (b3 - a53) * dt, vec_n, (b4 - a54) * dt, t1.data());
  O->apply(t2.data(), t1.data());
  vec_update(nd, 1.0, vec_np, b5 * dt, t1.data(), 0.0, nullptr);
}

// SSPRK(order 4, 8 stages), SSPRK::perform_time_step (time_integrators.cc:440-478)
// with the coefficients of initialize_coeffs (time_integrators.cc:726-795):
// u_s = sum_{l<s} A[s-1][l] u_l + dt B[s-1][l] M^-1 A(u_l), u_0 = vec_n,
// vec_np = u_8.  Rows are listed as (l, A, B) for the nonzero entries.
struct SspTerm {
  int l;
  double a, b;
};
static const SspTerm kSsp48[8][8] = {
    {{0, 1., 0.282318339066479}},
    {{0, 0.538569155333175, 0.}, {1, 0.461430844666825, 0.130270389660380}},
    {{0, 0.004485387460763, 0.003963092203460}, {2, 0.995514612539237, 0.281052031928487}},
    {{0, 0.164495299288580, 0.000038019518678}, {1, 0.016875060685979, 0.004764139104512},
     {3, 0.818629640025440, 0.231114160282572}},
    {{0, 0.426933682982668, 0.000019921336144}, {1, 0.157047028197878, 0.044337256156151},
     {2, 0.023164224070770, 0.006539685265423}, {4, 0.392855064748685, 0.110910189373703}},
    {{0, 0.082083400476958, 0.000000034006679}, {1, 0.000000039091042, 0.000000011036118},
     {2, 0.033974171137350, 0.009591531566657}, {3, 0.005505195713107, 0.001554217709960},
     {5, 0.878437193581543, 0.247998929466160}},
    {{0, 0.006736365648625, 0.013159891155054}, {1, 0.010581829625529, 0.002987444564164},
     {2, 0.009353386191951, 0.002640632454359}, {3, 0.101886062556838, 0.028764303955070},
     {4, 0.000023428364930, 0.000006614257074}, {6, 0.871418927612128, 0.246017544274548}},
    {{0, 0.071115287415749, 0.000000010647874}, {1, 0.018677648343953, 0.005273042658132},
     {2, 0.007902408660034, 0.002230994887525}, {3, 0.319384027162348, 0.090167968072837},
     {4, 0.007121989995845, 0.002010668386475}, {5, 0.001631615692736, 0.000460635032368},
     {7, 0.574167022729334, 0.162097880203691}}};
static const int kSsp48Terms[8] = {1, 2, 2, 3, 4, 5, 6, 7};

void ewo_ssprk_step(ewo_problem* p, double dt, double* vec_n, double* vec_np) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int64_t nd = (int64_t)O->n_dofs();
  std::vector<std::vector<double>> u(9, std::vector<double>(nd)), k(8, std::vector<double>(nd));
  u[0].assign(vec_n, vec_n + nd);
  for (int s = 1; s <= 8; ++s) {
    O->apply(u[s - 1].data(), k[s - 1].data());
    std::fill(u[s].begin(), u[s].end(), 0.0);
    for (int t = 0; t < kSsp48Terms[s - 1]; ++t) {
      const SspTerm& c = kSsp48[s - 1][t];
      vec_update(nd, 1.0, u[s].data(), c.a, u[c.l].data(), c.b * dt, k[c.l].data());
    }
  }
  std::copy(u[8].begin(), u[8].end(), vec_np);
}

// Time-integrated state of the first ADER step (local_apply_firstader_domain,
// wave_equation_operations.cc:939-957), written to T.
void ewo_ader_taylor(ewo_problem* p, double dt, const double* src, double* T) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  std::vector<double> d1;
  if (O->use_ader_post) {
    d1.resize(O->n_dofs());
    O->apply(src, d1.data());
  }
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < O->mesh.n_cells; ++c)
    O->ck_cell(c, src, O->use_ader_post ? d1.data() : nullptr, dt, T);
}

// WaveEquationOperationADER::apply_ader (wave_equation_operations.cc:1346-1381):
// dst = -M^{-1} A(T).
void ewo_apply_ader(ewo_problem* p, double dt, const double* src, double* dst) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  std::vector<double> T(O->n_dofs());
  ewo_ader_taylor(p, dt, src, T.data());
  O->apply(T.data(), dst, -1.0);
}

// ArbitraryHighOrderDG::perform_time_step (time_integrators.cc:37-50)
void ewo_ader_step(ewo_problem* p, double dt, const double* vec_n, double* vec_np) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  ewo_apply_ader(p, dt, vec_n, vec_np);
  const int64_t nd = (int64_t)O->n_dofs();
  for (int64_t i = 0; i < nd; ++i) vec_np[i] = -vec_np[i] + vec_n[i];
}

// WaveEquationOperationADERADCONFULL::apply_ader (wave_equation_operations.cc:689-735)
// followed by the ADER update: the Taylor series built from k+1 operator sweeps.
void ewo_aderadconfull_step(ewo_problem* p, double dt, const double* vec_n, double* vec_np) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int64_t nd = (int64_t)O->n_dofs();
  std::vector<double> acc(nd, 0.0), tv(nd), dst(nd);
  O->apply(vec_n, dst.data());
  for (int64_t i = 0; i < nd; ++i) {
    acc[i] = acc[i] - dt * dst[i];
    tv[i] = -dst[i];
  }
  double fac = -0.5 * dt * dt;
  for (int kk = 1; kk <= O->k; ++kk) {
    O->apply(tv.data(), dst.data());
    for (int64_t i = 0; i < nd; ++i) {
      acc[i] = acc[i] - fac * dst[i];
      tv[i] = -dst[i];
    }
    fac *= -dt / (kk + 2);
  }
  for (int64_t i = 0; i < nd; ++i) vec_np[i] = -acc[i] + vec_n[i];
}

// "error p post" against the reference's single-mode solution.
double ewo_post_error_reference(ewo_problem* p, const double* u, int modes, double t) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int dim = O->dim;
  return post_pressure_error(*O, u, [&](const double* x, double* ex) { exact_reference(dim, modes, x, t, ex); });
}

// L2 errors against the reference's single-mode solution: out = {err p, err u, |p|}.
void ewo_errors_reference(ewo_problem* p, const double* u, int modes, double t, double* out) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const int dim = O->dim;
  l2_errors(*O, u, [&](const double* x, double* ex) { exact_reference(dim, modes, x, t, ex); },
            out);
}

void ewo_errors_modes(ewo_problem* p, const double* u, int n_modes, const double* amp,
                      const int* kv, double t, double* out) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  ModeSet ms;
  ms.amp.assign(amp, amp + n_modes);
  ms.kv.assign(kv, kv + 3 * n_modes);
  const int dim = O->dim;
  l2_errors(*O, u, [&](const double* x, double* ex) { exact_membrane(dim, ms, x, t, ex); }, out);
}

// Replays the reference's time loop (explicit_wave.cc:549-813 with
// TimeControl, utilities.cc:31-95) for integrator 0 = LSRK45R2, 1 = clRK4,
// 2 = ADER, 3 = ADERADCONFULL, 4 = ExplEuler, 5 = LSRK33R2, 6 = LSRK45R3,
// 7 = LSRK59R2, 8 = SSPRK.  cfl is the Courant number as written in the
// parameter file (divided by k^1.5 here, parameters.cc:195).  Each output
// tick appends {time, step, err p, err u, |p|} to rows (capacity max_rows);
// returns the number of rows, or -1 on error.  dt_out receives the
// (unrounded) time step actually used.
int ewo_run_reference(ewo_problem* p, int integrator, double cfl, double final_time,
                      double tick, int modes, int max_time_steps, double* rows, int max_rows,
                      double* dt_out) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  const double dt = ewo_time_step(p, cfl / std::pow((double)O->k, 1.5));
  if (dt_out) *dt_out = dt;
  std::vector<double> sol(O->n_dofs()), tmp(O->n_dofs());
  ewo_project_reference(p, modes, 0.0, sol.data());
  int nrows = 0;
  double time = 0.0;
  unsigned step = 0;
  auto emit = [&]() {
    if (nrows >= max_rows) return;
    double e[3];
    ewo_errors_reference(p, sol.data(), modes, time, e);
    double* r = rows + 6 * nrows;
    r[0] = time;
    r[1] = step;
    r[2] = e[0];
    r[3] = e[1];
    r[4] = e[2];
    r[5] = ewo_post_error_reference(p, sol.data(), modes, time);
    ++nrows;
  };
  emit();
  // TimeControl::setup (utilities.cc:38-46): 0 means the number of steps of
  // the rounded step size
  if (max_time_steps == 0) {
    const double rounded = final_time / std::max(std::round(final_time / dt), 1.0);
    max_time_steps = (int)std::round(final_time / rounded);
  }
  while (!(time >= final_time || step > (unsigned)max_time_steps)) {
    ++step;
    time += dt;
    tmp.swap(sol);
    switch (integrator) {
      case 0: ewo_lsrk45_step(p, dt, tmp.data(), sol.data()); break;
      case 1: ewo_clrk4_step(p, dt, tmp.data(), sol.data()); break;
      case 2: ewo_ader_step(p, dt, tmp.data(), sol.data()); break;
      case 3: ewo_aderadconfull_step(p, dt, tmp.data(), sol.data()); break;
      case 4: ewo_expleuler_step(p, dt, tmp.data(), sol.data()); break;
      case 5: ewo_lsrk33_step(p, dt, tmp.data(), sol.data()); break;
      case 6: ewo_lsrk45r3_step(p, dt, tmp.data(), sol.data()); break;
      case 7: ewo_lsrk59_step(p, dt, tmp.data(), sol.data()); break;
      case 8: ewo_ssprk_step(p, dt, tmp.data(), sol.data()); break;
      default: g_last_error = "unknown integrator"; return -1;
    }
    if ((int)(time / tick) != (int)((time - dt) / tick)) emit();
  }
  return nrows;
}

// ---- extensions without a reference counterpart (point sources, receivers)

// Cell containing x and its reference coordinates (Newton on the
// multilinear map, after a bounding-box test).
static bool ewo_locate(const Oracle* O, const double* x, int64_t* cell, double* xi) {
  const int dim = O->dim, nv = 1 << dim;
  for (int64_t c = 0; c < O->mesh.n_cells; ++c) {
    const double* V = &O->mesh.vert[(size_t)c * nv * dim];
    bool in = true;
    for (int e = 0; e < dim && in; ++e) {
      double lo = 1e300, hi = -1e300;
      for (int v = 0; v < nv; ++v) {
        lo = std::min(lo, V[v * dim + e]);
        hi = std::max(hi, V[v * dim + e]);
      }
      if (x[e] < lo - 1e-12 || x[e] > hi + 1e-12) in = false;
    }
    if (!in) continue;
    double r[3] = {0.5, 0.5, 0.5};
    for (int it = 0; it < 50; ++it) {
      double y[3] = {0, 0, 0}, J[3][3], JiT[3][3];
      map_point(dim, V, r, y);
      jacobian(dim, V, r, J);
      inverse_transpose(dim, J, JiT);
      double step = 0.0;
      for (int e = 0; e < dim; ++e) {
        double d = 0.0;  // (J^{-1} (x - y))_e = sum_d JiT[d][e] (x-y)_d
        for (int dd = 0; dd < dim; ++dd) d += JiT[dd][e] * (x[dd] - y[dd]);
        r[e] += d;
        step += std::fabs(d);
      }
      if (step < 1e-15) break;
    }
    bool inside = true;
    for (int e = 0; e < dim; ++e)
      if (r[e] < -1e-10 || r[e] > 1 + 1e-10) inside = false;
    if (!inside) continue;
    *cell = c;
    for (int e = 0; e < dim; ++e) xi[e] = r[e];
    return true;
  }
  return false;
}

// Pressure of the DG field u at physical points (receivers): out[i].
int ewo_point_values(ewo_problem* p, const double* u, int n, const double* pts, double* out) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  for (int i = 0; i < n; ++i) {
    int64_t c;
    double xi[3] = {0, 0, 0};
    if (!ewo_locate(O, pts + i * O->dim, &c, xi)) {
      g_last_error = "point outside the mesh";
      return -1;
    }
    double v = 0.0;
    for (int q = 0; q < O->N; ++q) {
      int ii[3] = {0, 0, 0};
      O->point_index(q, ii);
      double w = 1.0;
      for (int e = 0; e < O->dim; ++e) w *= O->B.lag.value(ii[e], xi[e]);
      v += w * u[(size_t)c * O->F * O->N + O->dim * O->N + q];
    }
    out[i] = v;
  }
  return 0;
}

// LSRK45 step with a Ricker point source amp*(1-2a)exp(-a), a = pi^2 f0^2
// (t-delay)^2, added to the pressure equation at the stage times
// t + c_s dt: the term amp*r(t) phi_q(x_s) / JxW_q on the source cell.
int ewo_lsrk45_step_source(ewo_problem* p, double dt, double t, double* vec_n, double* vec_np,
                           const double* xs, double amp, double f0, double delay) {
  Oracle* O = reinterpret_cast<Oracle*>(p);
  int64_t cell;
  double xi[3] = {0, 0, 0};
  if (!ewo_locate(O, xs, &cell, xi)) {
    g_last_error = "source outside the mesh";
    return -1;
  }
  std::vector<double> w(O->N);
  for (int q = 0; q < O->N; ++q) {
    int ii[3] = {0, 0, 0};
    O->point_index(q, ii);
    double phi = 1.0, r[3] = {0, 0, 0};
    for (int e = 0; e < O->dim; ++e) {
      phi *= O->B.lag.value(ii[e], xi[e]);
      r[e] = O->B.rule.x[ii[e]];
    }
    double JiT[3][3];
    const double det = O->geom(cell, r, JiT);
    w[q] = phi / (det * O->W[q]);
  }
  const double a21 = 970286171893. / 4311952581923.;
  const double a32 = 6584761158862. / 12103376702013.;
  const double a43 = 2251764453980. / 15575788980749.;
  const double a54 = 26877169314380. / 34165994151039.;
  const double b1 = 1153189308089. / 22510343858157.;
  const double b2 = 1772645290293. / 4653164025191.;
  const double b3 = -1672844663538. / 4480602732383.;
  const double b4 = 2114624349019. / 3568978502595.;
  const double b5 = 5198255086312. / 14908931495163.;
  const double A[5] = {a21, a32, a43, a54, b5};
  const double Bm[5] = {b1 - a21, b2 - a32, b3 - a43, b4 - a54, 0.0};
  const double cs[5] = {0.0, a21, b1 + a32, b1 + b2 + a43, b1 + b2 + b3 + a54};
  const int64_t nd = (int64_t)O->n_dofs();
  std::vector<double> tmp(nd);
  double* in[5] = {vec_n, vec_n, vec_np, vec_n, vec_np};
  double* v2[5] = {vec_n, vec_np, vec_n, vec_np, vec_np};
  double* v3[5] = {vec_np, vec_n, vec_np, vec_n, vec_n};
  for (int st = 0; st < 5; ++st) {
    O->apply(in[st], tmp.data());
    const double ts = t + cs[st] * dt;
    const double aa = kPi * kPi * f0 * f0 * (ts - delay) * (ts - delay);
    const double r = amp * (1.0 - 2.0 * aa) * std::exp(-aa);
    for (int q = 0; q < O->N; ++q) tmp[(size_t)cell * O->F * O->N + O->dim * O->N + q] += r * w[q];
    ewo_rk_update(nd, A[st] * dt, Bm[st] * dt, st == 4, tmp.data(), v2[st], v3[st]);
  }
  return 0;
}

int ewo_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
