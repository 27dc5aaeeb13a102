// ew_cpu_cart.cpp -- CPU baseline for axis-aligned (Cartesian) meshes: the
// same operator and LowStorageRK45Reg2 step as ew_oracle.cpp, restated for
// speed on the host's cores.  Test infrastructure and timing baseline only
// (tests/, bench.py's CPU legs); nothing of the product calls it.
//
// On an axis-aligned cell the Jacobian is diag(h), so in direction e only u_e
// and p interact (evaluate_cell, wave_equation_operations.cc:424-456; the
// faces normal to e, evaluate_inner_face :480-551 and
// evaluate_boundary_face :569-629; the inverse mass matrix :633-661 is a
// division by the cell's quadrature weights).  Per (cell, direction, line):
//   k_u(i)  = bf / h_e (-rho^-1 sum_j D_ij p_j + sum_s l_i(s)/w_i F_u(s))
//   k_p(i) += bf / h_e ( rho c^2 sum_j D_ji w_j/w_i u_j + sum_s l_i(s)/w_i F_p(s))
// with the upwind fluxes F at both ends of the line.  The step fuses each
// operator application with the RKVectorUpdater arithmetic
// (time_integrators.cc:107-195, 235-283) in three FP64 registers, like the
// GPU FP64 path.  Sizes are compile-time per degree (k = 1..7) so that the
// line loops unroll; cells run in parallel (OpenMP).  (Laying each
// direction's lines out as [point][line] to vectorise across lines measured
// slower with the portable flags: the transposes cost more than 2-wide
// vectors gain.  So did blocks of four cells with the cell index innermost,
// the layout of the reference's vectorised cell batches: 2.8e8 against
// 4.1e8 DoF-updates/s on eight x86 cores, the strided per-cell loads and the
// block's larger working set costing more than the vectorised sums save.)
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

namespace {

constexpr int ipw(int b, int e) { return e == 0 ? 1 : b * ipw(b, e - 1); }

struct CartData {
  int dim = 0, np = 0;
  int64_t n_cells = 0;
  const int32_t* nbr = nullptr;
  std::vector<double> ih;       // [cell][dim] 1/h
  std::vector<double> rho, cc;  // [cell]
  std::vector<double> D, Dt, L0, L1, W0, W1;  // 1-D data: D[i*n+j], Dt[i*n+j] = D[j][i] w_j/w_i, l(0), l(1), l/w
};

template <int DIM, int NP>
void apply_stage(const CartData& C, const double* X, const double* A, double* Xo, double* Ao, double f1,
                 double f2, int mode, double bf) {
  constexpr int N = ipw(NP, DIM), F = DIM + 1, NL = ipw(NP, DIM - 1);
  double D[NP][NP], Dt[NP][NP], L0[NP], L1[NP], W0[NP], W1[NP];
  for (int i = 0; i < NP; ++i) {
    for (int j = 0; j < NP; ++j) {
      D[i][j] = C.D[i * NP + j];
      Dt[i][j] = C.Dt[i * NP + j];
    }
    L0[i] = C.L0[i];
    L1[i] = C.L1[i];
    W0[i] = C.W0[i];
    W1[i] = C.W1[i];
  }
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < C.n_cells; ++c) {
    const double* u = X + (size_t)c * F * N;
    double k[F * N];
    for (int q = 0; q < N; ++q) k[DIM * N + q] = 0.0;
    const double rho = C.rho[c], cs = C.cc[c];
    const double rho_inv = 1.0 / rho, rc2 = rho * cs * cs, tau_p = 1.0 / (cs * rho);
    for (int e = 0; e < DIM; ++e) {
      const int str = ipw(NP, e);
      const double ih = C.ih[c * DIM + e] * bf;
      const int nbs[2] = {C.nbr[c * 2 * DIM + 2 * e], C.nbr[c * 2 * DIM + 2 * e + 1]};
      for (int t = 0; t < NL; ++t) {
        // first point of line t along e
        int base = 0, tt = t, m = 1;
        for (int d = 0; d < DIM; ++d) {
          if (d != e) {
            base += (tt % NP) * m;
            tt /= NP;
          }
          m *= NP;
        }
        double xu[NP], xp[NP];
        for (int j = 0; j < NP; ++j) {
          xu[j] = u[e * N + base + j * str];
          xp[j] = u[DIM * N + base + j * str];
        }
        double tu[2] = {0.0, 0.0}, tp[2] = {0.0, 0.0};
        for (int j = 0; j < NP; ++j) {
          tu[0] += L0[j] * xu[j];
          tu[1] += L1[j] * xu[j];
          tp[0] += L0[j] * xp[j];
          tp[1] += L1[j] * xp[j];
        }
        double Fu[2], Fp[2];
        for (int s = 0; s < 2; ++s) {
          const double nrm = s ? 1.0 : -1.0;
          const double un_p = nrm * tu[s];
          const int nb = nbs[s];
          double lambda;
          if (nb >= 0) {
            // neighbour's traces on this face, l_j(1 - s)
            const double* um = X + (size_t)nb * F * N;
            const double* Lm = s ? L0 : L1;
            double vu = 0.0, vp = 0.0;
            for (int j = 0; j < NP; ++j) {
              vu += Lm[j] * um[e * N + base + j * str];
              vp += Lm[j] * um[DIM * N + base + j * str];
            }
            const double un_m = -nrm * vu;
            const double tau_m = 1.0 / (C.cc[nb] * C.rho[nb]);
            const double tau_inv = 1.0 / (tau_p + tau_m);
            lambda = tau_inv * (un_p + un_m + tau_p * tp[s] + tau_m * vp);
          } else {
            const int id = -nb;
            if (id == 1)
              lambda = un_p / tau_p + tp[s];
            else if (id == 3)
              lambda = tau_p / (tau_p + tau_p) * tp[s] + 1.0 / (tau_p + tau_p) * un_p;
            else
              lambda = 0.0;
          }
          Fu[s] = (tp[s] - lambda) * rho_inv * nrm;
          Fp[s] = rc2 * (-un_p + tau_p * (lambda - tp[s]));
        }
        for (int i = 0; i < NP; ++i) {
          double gp = 0.0, du = 0.0;
          for (int j = 0; j < NP; ++j) {
            gp += D[i][j] * xp[j];
            du += Dt[i][j] * xu[j];
          }
          const int q = base + i * str;
          k[e * N + q] = ih * (-rho_inv * gp + W0[i] * Fu[0] + W1[i] * Fu[1]);
          k[DIM * N + q] += ih * (rc2 * du + W0[i] * Fp[0] + W1[i] * Fp[1]);
        }
      }
    }
    // the two-register update (RKVectorUpdater) of this cell
    const size_t o = (size_t)c * F * N;
    if (mode == 0) {
      for (int q = 0; q < F * N; ++q) Ao[o + q] = k[q];
    } else if (mode == 1) {
      for (int q = 0; q < F * N; ++q) {
        const double x = A[o + q] + f1 * k[q];
        Xo[o + q] = x;
        Ao[o + q] = x + f2 * k[q];
      }
    } else {
      for (int q = 0; q < F * N; ++q) Ao[o + q] = A[o + q] + f1 * k[q];
    }
  }
}

using StageFn = void (*)(const CartData&, const double*, const double*, double*, double*, double, double,
                         int, double);

template <int DIM>
StageFn pick(int np) {
  switch (np) {
    case 2: return apply_stage<DIM, 2>;
    case 3: return apply_stage<DIM, 3>;
    case 4: return apply_stage<DIM, 4>;
    case 5: return apply_stage<DIM, 5>;
    case 6: return apply_stage<DIM, 6>;
    case 7: return apply_stage<DIM, 7>;
    case 8: return apply_stage<DIM, 8>;
    default: return nullptr;
  }
}

}  // namespace

extern "C" {

struct ewc_problem;

// Axis-aligned mesh: vertices [cell][2^dim][dim], neighbours [cell][2 dim]
// (negative: boundary id), per-cell speed and density; 1-D Gauss data of
// np = k + 1 points: weights w, derivative matrix D[i*np+j] = l_j'(x_i),
// traces l_j(0), l_j(1).  Returns NULL for a cell that is not a box or an
// unsupported degree.
ewc_problem* ewc_create(int dim, int np, int64_t n_cells, const double* vertices, const int32_t* nbr,
                        const double* speed, const double* density, const double* w, const double* D,
                        const double* L0, const double* L1) {
  if ((dim != 2 && dim != 3) || np < 2 || np > 8 || n_cells < 1) return nullptr;
  CartData* C = new CartData;
  C->dim = dim;
  C->np = np;
  C->n_cells = n_cells;
  C->nbr = nbr;
  const int nv = 1 << dim;
  C->ih.resize((size_t)n_cells * dim);
  C->rho.assign(density, density + n_cells);
  C->cc.assign(speed, speed + n_cells);
  for (int64_t c = 0; c < n_cells; ++c) {
    const double* V = vertices + (size_t)c * nv * dim;
    for (int v = 0; v < nv; ++v)
      for (int e = 0; e < dim; ++e) {
        const double ref = ((v >> e) & 1) ? V[(nv - 1) * dim + e] : V[e];
        if (V[v * dim + e] != ref) {
          delete C;
          return nullptr;
        }
      }
    for (int e = 0; e < dim; ++e) C->ih[c * dim + e] = 1.0 / (V[(nv - 1) * dim + e] - V[e]);
  }
  C->D.assign(D, D + np * np);
  C->Dt.resize(np * np);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) C->Dt[i * np + j] = D[j * np + i] * w[j] / w[i];
  C->L0.assign(L0, L0 + np);
  C->L1.assign(L1, L1 + np);
  C->W0.resize(np);
  C->W1.resize(np);
  for (int i = 0; i < np; ++i) {
    C->W0[i] = L0[i] / w[i];
    C->W1[i] = L1[i] / w[i];
  }
  return reinterpret_cast<ewc_problem*>(C);
}

void ewc_destroy(ewc_problem* p) { delete reinterpret_cast<CartData*>(p); }

// dst = M^-1 A(src)
int ewc_apply(ewc_problem* p, const double* src, double* dst) {
  const CartData* C = reinterpret_cast<const CartData*>(p);
  StageFn f = C->dim == 2 ? pick<2>(C->np) : pick<3>(C->np);
  if (!f) return -1;
  f(*C, src, nullptr, nullptr, dst, 0.0, 0.0, 0, 1.0);
  return 0;
}

// One LowStorageRK45Reg2 step (time_integrators.cc:235-283): vec_n = u^n in,
// vec_np = u^{n+1} out, vec_n clobbered; tmp is a third register of n_dofs.
int ewc_lsrk45_step(ewc_problem* p, double dt, double* vec_n, double* vec_np, double* tmp) {
  const CartData* C = reinterpret_cast<const CartData*>(p);
  StageFn f = C->dim == 2 ? pick<2>(C->np) : pick<3>(C->np);
  if (!f) return -1;
  const double a21 = 970286171893. / 4311952581923., a32 = 6584761158862. / 12103376702013.;
  const double a43 = 2251764453980. / 15575788980749., a54 = 26877169314380. / 34165994151039.;
  const double b1 = 1153189308089. / 22510343858157., b2 = 1772645290293. / 4653164025191.;
  const double b3 = -1672844663538. / 4480602732383., b4 = 2114624349019. / 3568978502595.;
  const double b5 = 5198255086312. / 14908931495163.;
  const double f1[5] = {a21 * dt, a32 * dt, a43 * dt, a54 * dt, b5 * dt};
  const double f2[5] = {(b1 - a21) * dt, (b2 - a32) * dt, (b3 - a43) * dt, (b4 - a54) * dt, 0.0};
  double *N = vec_n, *P = vec_np, *T = tmp;
  // registers (stage input X, accumulator A, next input, next accumulator)
  double* X[5] = {N, T, P, N, T};
  double* A[5] = {N, P, N, T, P};
  double* Xo[5] = {T, P, N, T, nullptr};
  double* Ao[5] = {P, N, T, P, P};
  for (int s = 0; s < 5; ++s) f(*C, X[s], A[s], Xo[s], Ao[s], f1[s], f2[s], s < 4 ? 1 : 2, 1.0);
  return 0;
}

}  // extern "C"
