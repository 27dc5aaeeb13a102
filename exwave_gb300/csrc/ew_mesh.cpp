// ew_mesh.cpp -- host-side structured mesh generator (the problem
// definition of the reference, input_parameters.h:42-88, with the vertex
// transform of the 3-D curved configuration and per-face boundary ids).
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/exwave_gb300.h"
#include "ew_basis.h"

namespace {

int64_t ipow64(int64_t b, int e) {
  int64_t r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

bool valid(const ew_hypercube_desc* d) {
  if (!d || (d->dim != 2 && d->dim != 3) || d->n_intervals < 1 || d->n_refinements < 0 ||
      d->n_refinements > 12 || (d->transform != 0 && d->transform != 1))
    return false;
  for (int f = 0; f < 2 * d->dim; ++f)
    if (d->boundary_ids[f] < 1 || d->boundary_ids[f] > 3) return false;
  const int64_t m = (int64_t)d->n_intervals << d->n_refinements;
  return ipow64(m, d->dim) <= 0x7fffffff;
}

void multilinear(int dim, const double* V, const double* xi, double* x) {
  for (int i = 0; i < dim; ++i) x[i] = 0.0;
  for (int v = 0; v < (1 << dim); ++v) {
    double phi = 1.0;
    for (int e = 0; e < dim; ++e) phi *= ((v >> e) & 1) ? xi[e] : 1.0 - xi[e];
    for (int i = 0; i < dim; ++i) x[i] += V[v * dim + i] * phi;
  }
}

// Per-cell tensor-product interpolation: dst[c][f] = (M x M (x M)) src[c][f]
// with the 1-D matrix M (n x n, row q = output point), points lexicographic.
void tensor_interp(int dim, int n, int64_t n_cells, int n_fields, const std::vector<double>& M,
                   const double* src, double* dst) {
  const int64_t N = ipow64(n, dim);
  std::vector<double> a((size_t)N), b((size_t)N);
  for (int64_t cf = 0; cf < n_cells * n_fields; ++cf) {
    const double* in = src + cf * N;
    for (int64_t i = 0; i < N; ++i) a[i] = in[i];
    for (int e = 0; e < dim; ++e) {
      const int64_t str = ipow64(n, e);
      for (int64_t i = 0; i < N; ++i) {
        const int64_t j = (i / str) % n;      // this point's index along e
        const int64_t base = i - j * str;     // the line's first point
        double v = 0.0;
        for (int l = 0; l < n; ++l) v += M[(size_t)j * n + l] * a[base + l * str];
        b[i] = v;
      }
      a.swap(b);
    }
    double* out = dst + cf * N;
    for (int64_t i = 0; i < N; ++i) out[i] = a[i];
  }
}

// 1-D interpolation matrix from values at `from` to values at `to`
std::vector<double> interp_matrix(const std::vector<double>& from, const std::vector<double>& to) {
  const int n = (int)from.size();
  std::vector<double> M((size_t)n * n);
  for (int q = 0; q < n; ++q)
    for (int j = 0; j < n; ++j) M[(size_t)q * n + j] = ew::lagrange(from, j, to[q]);
  return M;
}

int nodal_convert(int dim, int degree, int64_t n_cells, int n_fields, const double* nodes,
                  const double* src, double* dst, bool to_gauss) {
  if ((dim != 2 && dim != 3) || degree < 1 || degree > 15 || n_cells < 0 || n_fields < 1 || !nodes)
    return EW_ERR_INVALID;
  if (n_cells > 0 && (!src || !dst || src == dst)) return EW_ERR_INVALID;
  const int n = degree + 1;
  std::vector<double> y(nodes, nodes + n);
  for (int i = 0; i < n; ++i) {
    if (!std::isfinite(y[i])) return EW_ERR_INVALID;
    for (int j = 0; j < i; ++j)
      if (!(std::fabs(y[i] - y[j]) > 1e-12)) return EW_ERR_INVALID;  // distinct nodes
  }
  const std::vector<double> g = ew::gauss_rule(n).x;
  tensor_interp(dim, n, n_cells, n_fields, to_gauss ? interp_matrix(y, g) : interp_matrix(g, y), src,
                dst);
  return EW_OK;
}

}  // namespace

extern "C" {

int ew_nodal_to_gauss(int32_t dim, int32_t degree, int64_t n_cells, int32_t n_fields,
                      const double* nodes, const double* src, double* dst) {
  return nodal_convert(dim, degree, n_cells, n_fields, nodes, src, dst, true);
}

int ew_gauss_to_nodal(int32_t dim, int32_t degree, int64_t n_cells, int32_t n_fields,
                      const double* nodes, const double* src, double* dst) {
  return nodal_convert(dim, degree, n_cells, n_fields, nodes, src, dst, false);
}


int64_t ew_hypercube_n_cells(const ew_hypercube_desc* d) {
  if (!valid(d)) return -1;
  return ipow64((int64_t)d->n_intervals << d->n_refinements, d->dim);
}

int ew_hypercube_mesh(const ew_hypercube_desc* d, double* vertices, int32_t* neighbors) {
  if (!valid(d) || !vertices || !neighbors) return EW_ERR_INVALID;
  const double pi = 3.14159265358979323846;
  const int dim = d->dim, n = d->n_intervals, sub = 1 << d->n_refinements;
  const int M = n * sub, nvc = n + 1, nv = 1 << dim;
  // transformed coarse vertices
  std::vector<double> cv((size_t)ipow64(nvc, dim) * dim);
  for (int64_t idx = 0; idx < ipow64(nvc, dim); ++idx) {
    double p[3] = {0, 0, 0};
    int64_t t = idx;
    for (int e = 0; e < dim; ++e) {
      p[e] = (double)(t % nvc) / n;
      t /= nvc;
    }
    if (d->transform == 0) {
      double s = d->transform_factor;
      for (int e = 0; e < dim; ++e) s *= std::sin(pi * p[e]);
      p[0] = p[0] + s;
    } else {
      double s = d->transform_factor;
      for (int e = 0; e < dim; ++e) s *= std::sin(2.0 * pi * p[e]);
      for (int e = 0; e < dim; ++e) p[e] = p[e] + s;
    }
    for (int e = 0; e < dim; ++e) cv[idx * dim + e] = p[e];
  }
  const int64_t n_cells = ipow64(M, dim);
  for (int64_t c = 0; c < n_cells; ++c) {
    int ic[3] = {0, 0, 0};
    int64_t t = c;
    for (int e = 0; e < dim; ++e) {
      ic[e] = (int)(t % M);
      t /= M;
    }
    for (int v = 0; v < nv; ++v) {
      int cc[3] = {0, 0, 0};
      double xi[3] = {0, 0, 0};
      for (int e = 0; e < dim; ++e) {
        const int g = ic[e] + ((v >> e) & 1);
        cc[e] = g / sub < n - 1 ? g / sub : n - 1;
        xi[e] = (double)(g - cc[e] * sub) / sub;
      }
      double V[8 * 3];
      for (int w = 0; w < nv; ++w) {
        int64_t idx = 0, str = 1;
        for (int e = 0; e < dim; ++e) {
          idx += (cc[e] + ((w >> e) & 1)) * str;
          str *= nvc;
        }
        for (int e = 0; e < dim; ++e) V[w * dim + e] = cv[idx * dim + e];
      }
      multilinear(dim, V, xi, vertices + ((size_t)c * nv + v) * dim);
    }
    int64_t str = 1;
    for (int e = 0; e < dim; ++e) {
      neighbors[c * 2 * dim + 2 * e] = ic[e] > 0 ? (int32_t)(c - str) : -d->boundary_ids[2 * e];
      neighbors[c * 2 * dim + 2 * e + 1] =
          ic[e] < M - 1 ? (int32_t)(c + str) : -d->boundary_ids[2 * e + 1];
      str *= M;
    }
  }
  return EW_OK;
}

}  // extern "C"
