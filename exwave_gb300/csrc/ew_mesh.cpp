// ew_mesh.cpp -- host-side structured mesh generator (the problem
// definition of the reference, input_parameters.h:42-88, with the vertex
// transform of the 3-D curved configuration and per-face boundary ids).
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/exwave_gb300.h"

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

}  // namespace

extern "C" {

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
