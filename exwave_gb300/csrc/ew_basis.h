// ew_basis.h -- host-side 1D collocation data: Gauss rules on [0,1], the
// Lagrange basis on the Gauss points, derivative matrices, face
// interpolation vectors and the ADER degree-reduction operators.
#pragma once

#include <cmath>
#include <vector>

namespace ew {

struct GaussRule {
  std::vector<double> x, w;
};

// Gauss-Legendre rule with n points on [0,1] (weights sum to one).  Newton
// iteration on P_n from Chebyshev-like starting values; nodes mirrored so
// that x[n-1-i] = 1 - x[i].
inline GaussRule gauss_rule(int n) {
  GaussRule r;
  r.x.assign(n, 0.0);
  r.w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double t = std::cos(pi * (i + 0.75) / (n + 0.5));
    double pn = 0.0, dpn = 1.0;
    for (int it = 0; it < 100; ++it) {
      double a = 1.0, b = t;  // P_0, P_1
      for (int k = 2; k <= n; ++k) {
        const double c = ((2.0 * k - 1.0) * t * b - (k - 1.0) * a) / k;
        a = b;
        b = c;
      }
      pn = (n == 1) ? t : b;
      const double pm = (n == 1) ? 1.0 : a;
      dpn = (n == 1) ? 1.0 : n * (t * pn - pm) / (t * t - 1.0);
      const double step = pn / dpn;
      t -= step;
      if (std::fabs(step) < 1e-17) break;
    }
    {
      double a = 1.0, b = t;
      for (int k = 2; k <= n; ++k) {
        const double c = ((2.0 * k - 1.0) * t * b - (k - 1.0) * a) / k;
        a = b;
        b = c;
      }
      pn = (n == 1) ? t : b;
      const double pm = (n == 1) ? 1.0 : a;
      dpn = (n == 1) ? 1.0 : n * (t * pn - pm) / (t * t - 1.0);
    }
    const double w = 1.0 / ((1.0 - t * t) * dpn * dpn);  // half of 2/(...)
    r.x[i] = 0.5 * (1.0 - t);
    r.x[n - 1 - i] = 0.5 * (1.0 + t);
    r.w[i] = w;
    r.w[n - 1 - i] = w;
  }
  if (n % 2 == 1) r.x[n / 2] = 0.5;
  return r;
}

inline double lagrange(const std::vector<double>& y, int j, double x) {
  double v = 1.0;
  for (size_t m = 0; m < y.size(); ++m)
    if ((int)m != j) v *= (x - y[m]) / (y[j] - y[m]);
  return v;
}

inline double lagrange_deriv(const std::vector<double>& y, int j, double x) {
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

// Basis table of NP points with all ADER levels, laid out as the device code
// expects (ew_device.cuh: level r has m = NP - 2r points: x, w, D, L0, L1 and,
// for r >= 1, P (m x (m+2)) = weighted projection from level r-1 and
// E ((m+2) x m) = interpolation back).  The projection is the one the
// reference builds into shape_hessians_eo (wave_equation_operations.cc:276-315):
// P[i][q] = l_i^{low}(x_q^{high}) w_q^{high} / w_i^{low}.
inline std::vector<double> basis_table(int NP) {
  std::vector<double> out;
  GaussRule prev;
  for (int r = 0; NP - 2 * r >= 1; ++r) {
    const int m = NP - 2 * r;
    GaussRule g = gauss_rule(m);
    for (int i = 0; i < m; ++i) out.push_back(g.x[i]);
    for (int i = 0; i < m; ++i) out.push_back(g.w[i]);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) out.push_back(lagrange_deriv(g.x, j, g.x[i]));
    for (int j = 0; j < m; ++j) out.push_back(lagrange(g.x, j, 0.0));
    for (int j = 0; j < m; ++j) out.push_back(lagrange(g.x, j, 1.0));
    if (r > 0) {
      const int mp = m + 2;
      for (int i = 0; i < m; ++i)
        for (int q = 0; q < mp; ++q)
          out.push_back(lagrange(g.x, i, prev.x[q]) * prev.w[q] / g.w[i]);
      for (int q = 0; q < mp; ++q)
        for (int i = 0; i < m; ++i) out.push_back(lagrange(g.x, i, prev.x[q]));
    }
    prev = g;
  }
  return out;
}

}  // namespace ew
