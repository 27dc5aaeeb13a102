// ew_kernels.cuh -- the hot-path kernels, templated on dimension, points
// per direction (NP = k+1), compute precision and storage types.
//
//  stage_kernel : one launch = the whole operator M^{-1} A(X) of a stage
//                 (cell term, element-centric inner faces, boundary faces,
//                 inverse mass) fused with the epilogue of the integrator:
//                 plain result (WaveEquationOperation::apply), the two-register
//                 LSRK update (RKVectorUpdater) or the ADER update
//                 (ArbitraryHighOrderDG).
//  ck_kernel    : the ADER Taylor / Cauchy-Kovalevskaya time integral of
//                 each cell (WaveEquationOperationADER::integrate_taylor_cauchykovalewski),
//                 optionally starting from the full DG time derivative
//                 (use_ader_post), fused with the operator for that case.
//
// Thread mapping: one thread per Gauss point, CB cells per CTA, a
// grid-stride loop over a work list of cell blocks (one solve or many).
// Each CTA stages its cells' input in shared memory; a face reads the
// neighbour's values along the lines normal to the face from shared memory
// when the neighbour is in the same block and from L2 otherwise, so each
// vector is streamed from HBM about once per stage.
#pragma once

#include <type_traits>

#include "ew_ff.cuh"

namespace ew {

template <int DIM, int NP, bool CART>
struct Shape {
  static constexpr int N = ipow_c(NP, DIM);
  static constexpr int NF = ipow_c(NP, DIM - 1);
  static constexpr int F = DIM + 1;
  static constexpr int NV = 1 << DIM;
  static constexpr int FF = CART ? 2 : DIM + 1;   // flux values kept per face point
  static constexpr int GEO = CART ? DIM : NV * DIM;
  static constexpr int BAS = (basis_total(NP) + 3) & ~3;
};

// Shared-memory layout in units of Real.
template <int DIM, int NP, bool CART>
struct OpSmem {
  using S = Shape<DIM, NP, CART>;
  int basis, X, G, Fl, geo, mat, end;
  __host__ __device__ explicit OpSmem(int CB) {
    basis = 0;
    X = S::BAS;
    G = X + CB * S::F * S::N;
    Fl = G + CB * DIM * S::N;
    geo = Fl + CB * 2 * DIM * S::FF * S::NF;
    mat = geo + CB * S::GEO;
    end = (mat + CB * 4 + 3) & ~3;
  }
};

template <int DIM, int NP, bool CART>
struct CkSmem {
  using S = Shape<DIM, NP, CART>;
  OpSmem<DIM, NP, CART> op;
  int Sv, T1, T2, C[8], J, P, PG, PM, end;
  // in_words: Real-sized words per stored input value (2 for FP64 input to
  // the FP32 kernel, else 1)
  __host__ __device__ CkSmem(int CB, int in_words) : op(CB) {
    // J: inverse-transpose Jacobians at the level-0 points, [cell][DIM*DIM][point]
    J = op.end;
    Sv = J + (CART ? 0 : CB * DIM * DIM * S::N);
    T1 = Sv + CB * S::F * S::N;
    T2 = T1 + CB * S::F * S::N;
    int o = T2 + CB * S::F * S::N;
    for (int r = 0; r < 8; ++r) C[r] = o;
    for (int r = 1; r < n_levels(NP); ++r) {
      C[r] = o;
      o += CB * S::F * ipow_c(NP - 2 * r, DIM);
    }
    // P, PG, PM: the next work item's input values (as stored), geometry and
    // materials, copied asynchronously while the current item is computed
    P = (o + 3) & ~3;
    PG = P + CB * S::F * S::N * in_words;
    PM = PG + CB * S::GEO;
    end = (PM + CB * 4 + 3) & ~3;
  }
};

template <typename Real, typename T>
__device__ __forceinline__ Real to_real(T v) {
  if constexpr (std::is_same<Real, T>::value) {
    return v;
  } else if constexpr (sizeof(Real) == 4 && sizeof(T) == 8) {
    return f64_to_f32(v);
  } else if constexpr (sizeof(Real) == 8 && !std::is_floating_point<Real>::value) {
    // float-float from FP64: the exact pair; from FP32: the value
    if constexpr (std::is_same<T, double>::value) {
      float hi, lo;
      f64_split(v, hi, lo);
      return Real(hi, lo);
    } else {
      return Real(v);
    }
  } else {
    return static_cast<Real>(v);
  }
}

__device__ __forceinline__ int dir_stride(int e, int NP) { return e == 0 ? 1 : (e == 1 ? NP : NP * NP); }

// Copy the input of the block's cells, their geometry and materials into
// shared memory.
template <int DIM, int NP, typename Real, typename InT, bool CART>
__device__ __forceinline__ void load_block(const SolveDesc& sd, int cell_begin, int nc, Real* sX,
                                           Real* sGeo, Real* sMat) {
  using S = Shape<DIM, NP, CART>;
  const InT* X = static_cast<const InT*>(sd.X) + (size_t)cell_begin * S::F * S::N;
  const int total = nc * S::F * S::N;
  for (int i = threadIdx.x; i < total; i += blockDim.x) sX[i] = to_real<Real>(load_nc(X + i));
  const Real* G = static_cast<const Real*>(sd.geo) + (size_t)cell_begin * S::GEO;
  for (int i = threadIdx.x; i < nc * S::GEO; i += blockDim.x) sGeo[i] = load_nc(G + i);
  const Real* M = static_cast<const Real*>(sd.mat) + (size_t)cell_begin * 4;
  for (int i = threadIdx.x; i < nc * 4; i += blockDim.x) sMat[i] = load_nc(M + i);
}

// Cell term at point q of local cell cl: returns the velocity part
// (already divided by JxW) and 1/JxW; writes the contravariant pressure
// flux G_e = bf rho c^2 JxW (J^{-T} u)_e to sG.  evaluate_cell,
// wave_equation_operations.cc:424-456.
template <int DIM, int NP, typename Real, bool CART>
__device__ __forceinline__ void op_cell(const Real* sB, const Real* sX, Real* sG, const Real* sGeo,
                                        const Real* sMat, int cl, int q, Real bf, Real* Ru,
                                        Real& inv_jxw) {
  using S = Shape<DIM, NP, CART>;
  const Level<Real> L = get_level(sB, NP, 0);
  int i[3] = {0, 0, 0};
  split_point<DIM, NP>(q, i);
  const Real* x = sX + cl * S::F * S::N;
  const Real* p = x + DIM * S::N;
  Real gxi[DIM];
#pragma unroll
  for (int e = 0; e < DIM; ++e) {
    const int str = ipow_c(NP, e);
    const Real* row = L.D + i[e] * NP;
    const Real* line = p + q - i[e] * str;
    Real s = Real(0);
#pragma unroll
    for (int a = 0; a < NP; ++a) s += row[a] * line[a * str];
    gxi[e] = s;
  }
  Real xi[DIM];
  Real W = Real(1);
#pragma unroll
  for (int e = 0; e < DIM; ++e) {
    xi[e] = L.x[i[e]];
    W *= L.w[i[e]];
  }
  Real JiT[DIM][DIM];
  const Real det = cell_geom<DIM, Real, CART>(sGeo + cl * S::GEO, xi, JiT);
  const Real jxw = det * W;
  inv_jxw = Real(1) / jxw;
  const Real rho = sMat[4 * cl], c = sMat[4 * cl + 1];
  const Real fu = -bf / rho;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    Real g = Real(0);
#pragma unroll
    for (int e = 0; e < DIM; ++e) g += JiT[d][e] * gxi[e];
    Ru[d] = fu * g;
  }
  const Real fp = bf * rho * c * c * jxw;
#pragma unroll
  for (int e = 0; e < DIM; ++e) {
    Real s = Real(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) s += JiT[d][e] * x[d * S::N + q];
    sG[cl * DIM * S::N + e * S::N + q] = fp * s;
  }
}

// Flux at face point fp of the block (all faces of all cells of the block),
// times the face JxW, into sFl.  evaluate_inner_face (wave_equation_operations.cc:480-551)
// seen from this cell's side, and evaluate_boundary_face (569-629).
template <int DIM, int NP, typename Real, typename InT, bool CART>
__device__ __forceinline__ void op_face(const Real* sB, const Real* sX, Real* sFl, const Real* sGeo,
                                        const Real* sMat, const SolveDesc& sd, int cell_begin,
                                        int nc, int fp, Real bf, int* err) {
  using S = Shape<DIM, NP, CART>;
  constexpr int F = S::F, N = S::N, NF = S::NF;
  const Level<Real> L = get_level(sB, NP, 0);
  const int cl = fp / (2 * DIM * NF);
  const int rem = fp - cl * 2 * DIM * NF;
  const int f = rem / NF;
  const int t = rem - f * NF;
  const int e = f >> 1, s = f & 1;
  int ti[3] = {0, 0, 0};
  const int q0 = face_base<DIM, NP>(e, t, ti);
  const int str = dir_stride(e, NP);
  const Real* Ls = s ? L.L1 : L.L0;
  const Real* Lm = s ? L.L0 : L.L1;
  const Real* x = sX + cl * F * N;
  const Real sgn = s ? Real(1) : Real(-1);

  // own trace
  Real vp[F];
#pragma unroll
  for (int fld = 0; fld < F; ++fld) {
    vp[fld] = Real(0);
    if (CART && fld != e && fld != DIM) continue;
    Real a = Real(0);
#pragma unroll
    for (int j = 0; j < NP; ++j) a += Ls[j] * x[fld * N + q0 + j * str];
    vp[fld] = a;
  }
  // normal and face JxW
  Real nrm[DIM];
  Real jxw_f;
  if constexpr (CART) {
    const Real* h = sGeo + cl * S::GEO;
    Real area = Real(1);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      nrm[d] = (d == e) ? sgn : Real(0);
      if (d != e) area *= h[d] * L.w[ti[d]];
    }
    jxw_f = area;
  } else {
    Real xi[DIM];
    Real wt = Real(1);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      if (d == e) {
        xi[d] = s ? Real(1) : Real(0);
      } else {
        xi[d] = L.x[ti[d]];
        wt *= L.w[ti[d]];
      }
    }
    Real JiT[DIM][DIM];
    const Real det = geom_general<DIM, Real>(sGeo + cl * S::GEO, xi, JiT);
    Real len2 = Real(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      nrm[d] = sgn * JiT[d][e];
      len2 += nrm[d] * nrm[d];
    }
    const Real len = real_sqrt(len2);
    const Real il = Real(1) / len;
#pragma unroll
    for (int d = 0; d < DIM; ++d) nrm[d] *= il;
    jxw_f = wt * real_fabs(det) * len;
  }
  const Real rho = sMat[4 * cl], c = sMat[4 * cl + 1];
  const Real rho_inv = Real(1) / rho, c_sq = c * c;
  const Real tau_p = Real(1) / (c * rho);
  Real un_p = Real(0);
#pragma unroll
  for (int d = 0; d < DIM; ++d) un_p += vp[d] * nrm[d];

  const int cell = cell_begin + cl;
  int nb = sd.nbr[(size_t)cell * 2 * DIM + f];
  Real lambda;
  Real tau_here = tau_p;
  if (nb >= 0) {
    if (nb >= sd.n_cells) {
      atomicOr(err, ERR_BAD_NEIGHBOR);
      nb = cell;
    }
    Real vm[F];
    Real rho_m, c_m;
    const int nl = nb - cell_begin;
    if (nl >= 0 && nl < nc) {
      const Real* xm = sX + nl * F * N;
#pragma unroll
      for (int fld = 0; fld < F; ++fld) {
        vm[fld] = Real(0);
        if (CART && fld != e && fld != DIM) continue;
        Real a = Real(0);
#pragma unroll
        for (int j = 0; j < NP; ++j) a += Lm[j] * xm[fld * N + q0 + j * str];
        vm[fld] = a;
      }
      rho_m = sMat[4 * nl];
      c_m = sMat[4 * nl + 1];
    } else {
      const InT* xm = static_cast<const InT*>(sd.X) + (size_t)nb * F * N;
#pragma unroll
      for (int fld = 0; fld < F; ++fld) {
        vm[fld] = Real(0);
        if (CART && fld != e && fld != DIM) continue;
        Real a = Real(0);
#pragma unroll
        for (int j = 0; j < NP; ++j) a += Lm[j] * to_real<Real>(load_nc(xm + fld * N + q0 + j * str));
        vm[fld] = a;
      }
      const Real* M = static_cast<const Real*>(sd.mat);
      rho_m = load_nc(M + 4 * (size_t)nb);
      c_m = load_nc(M + 4 * (size_t)nb + 1);
    }
    Real un_m = Real(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) un_m -= vm[d] * nrm[d];
    const Real tau_m = Real(1) / (c_m * rho_m);
    const Real tau_inv = Real(1) / (tau_p + tau_m);
    lambda = tau_inv * (un_p + un_m + tau_p * vp[DIM] + tau_m * vm[DIM]);
  } else {
    const int id = -nb;
    if (id == EW_BC_SOFT_WALL_ID) {
      lambda = un_p / tau_p + vp[DIM];
    } else if (id == EW_BC_ABSORBING_ID) {
      const Real tsum = tau_p + Real(1) / (c * rho);
      lambda = tau_p / tsum * vp[DIM] + Real(1) / tsum * un_p;
    } else {
      if (id != EW_BC_HARD_WALL_ID) atomicOr(err, ERR_BAD_BOUNDARY_ID);
      lambda = Real(0);
    }
  }
  const Real scale = bf * jxw_f;
  const Real pd = (vp[DIM] - lambda) * rho_inv * scale;
  const Real fpres = c_sq * rho * (-un_p + tau_here * (lambda - vp[DIM])) * scale;
  Real* out = sFl + (cl * 2 * DIM + f) * S::FF * NF + t;
  if constexpr (CART) {
    out[0] = pd * nrm[e];
    out[NF] = fpres;
  } else {
#pragma unroll
    for (int d = 0; d < DIM; ++d) out[d * NF] = pd * nrm[d];
    out[DIM * NF] = fpres;
  }
}

// Gather of the cell term's pressure part, the face lifts and the inverse
// mass at point q: k = M^{-1} A(X) at that point (inverse mass:
// local_apply_mass_matrix, wave_equation_operations.cc:633-661).
template <int DIM, int NP, typename Real, bool CART>
__device__ __forceinline__ void op_collect(const Real* sB, const Real* sG, const Real* sFl, int cl,
                                           int q, const Real* Ru, Real inv_jxw, Real* k) {
  using S = Shape<DIM, NP, CART>;
  constexpr int N = S::N, NF = S::NF;
  const Level<Real> L = get_level(sB, NP, 0);
  int i[3] = {0, 0, 0};
  split_point<DIM, NP>(q, i);
  Real rp = Real(0);
#pragma unroll
  for (int e = 0; e < DIM; ++e) {
    const int str = ipow_c(NP, e);
    const Real* g = sG + cl * DIM * N + e * N + q - i[e] * str;
#pragma unroll
    for (int a = 0; a < NP; ++a) rp += L.D[a * NP + i[e]] * g[a * str];
  }
  Real lift[DIM + 1];
#pragma unroll
  for (int fld = 0; fld <= DIM; ++fld) lift[fld] = Real(0);
#pragma unroll
  for (int e = 0; e < DIM; ++e) {
    const int t = face_index<DIM, NP>(i, e);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const Real l = s ? L.L1[i[e]] : L.L0[i[e]];
      const Real* fl = sFl + (cl * 2 * DIM + 2 * e + s) * S::FF * NF + t;
      if constexpr (CART) {
        lift[e] += l * fl[0];
        lift[DIM] += l * fl[NF];
      } else {
#pragma unroll
        for (int fld = 0; fld <= DIM; ++fld) lift[fld] += l * fl[fld * NF];
      }
    }
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) k[d] = Ru[d] + lift[d] * inv_jxw;
  k[DIM] = (rp + lift[DIM]) * inv_jxw;
}

template <typename Real>
__device__ __forceinline__ void load_basis(const void* basis, Real* sB, int n) {
  const Real* b = static_cast<const Real*>(basis);
  for (int i = threadIdx.x; i < n; i += blockDim.x) sB[i] = b[i];
}

__device__ __forceinline__ const SolveDesc& pick(const LaunchArgs& La, int solve) {
  return La.solves ? La.solves[solve] : La.single;
}

// ============================================================ stage kernel
template <int DIM, int NP, typename Real, typename InT, typename OutT, bool CART>
__global__ void __launch_bounds__(512) stage_kernel(const LaunchArgs La) {
  using S = Shape<DIM, NP, CART>;
  constexpr int F = S::F, N = S::N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sm = reinterpret_cast<Real*>(smem_raw);
  const int CB = La.cells_per_block;
  const OpSmem<DIM, NP, CART> lay(CB);
  Real* sB = sm + lay.basis;
  Real* sX = sm + lay.X;
  Real* sG = sm + lay.G;
  Real* sFl = sm + lay.Fl;
  Real* sGeo = sm + lay.geo;
  Real* sMat = sm + lay.mat;
  // points per thread: one (CB cells of at most 512 points each), or, for a
  // cell of more points (3-D, degree 8 and above), several, one cell per block
  constexpr int PPT = (N + 511) / 512;
  if ((int)blockDim.x * PPT < CB * N || (PPT > 1 && CB != 1)) {
    if (threadIdx.x == 0) atomicOr(La.err, ERR_BAD_LAUNCH);
    return;
  }
  load_basis<Real>(La.basis, sB, basis_total(NP));

  for (int w = blockIdx.x; w < La.n_work; w += gridDim.x) {
    const WorkItem wi = La.work[w];
    const SolveDesc sd = pick(La, wi.solve);  // by value: no reloads after stores
    const int nc = wi.n_cells;
    __syncthreads();  // previous item done with shared memory; basis loaded
    load_block<DIM, NP, Real, InT, CART>(sd, wi.cell_begin, nc, sX, sGeo, sMat);
    __syncthreads();
    const Real bf = static_cast<Real>(sd.bf);
    Real Ru[PPT][DIM];
    Real inv_jxw[PPT];
#pragma unroll
    for (int r = 0; r < PPT; ++r) {
      const int idx = threadIdx.x + r * blockDim.x;
      const int cl = idx / N;
      inv_jxw[r] = Real(1);
      if (cl < nc) op_cell<DIM, NP, Real, CART>(sB, sX, sG, sGeo, sMat, cl, idx - cl * N, bf, Ru[r], inv_jxw[r]);
    }
    for (int fp = threadIdx.x; fp < nc * 2 * DIM * S::NF; fp += blockDim.x)
      op_face<DIM, NP, Real, InT, CART>(sB, sX, sFl, sGeo, sMat, sd, wi.cell_begin, nc, fp, bf,
                                        La.err);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PPT; ++r) {
    const int idx = threadIdx.x + r * blockDim.x;
    const int cl = idx / N;
    const int q = idx - cl * N;
    if (cl >= nc) continue;
    Real k[F];
    op_collect<DIM, NP, Real, CART>(sB, sG, sFl, cl, q, Ru[r], inv_jxw[r], k);

    const size_t g0 = ((size_t)wi.cell_begin + cl) * F * N + q;
    const int mode = sd.mode;
    if (mode == MODE_APPLY) {
#pragma unroll
      for (int fld = 0; fld < F; ++fld) {
        if constexpr (is_f64_v<Real>)
          sd.Aout[g0 + fld * N] = k[fld];
        else if constexpr (is_ff_v<Real>)
          sd.Aout[g0 + fld * N] = f32_to_f64(k[fld].hi) + f32_to_f64(k[fld].lo);
        else
          sd.Aout[g0 + fld * N] = f32_to_f64(k[fld]);
      }
    } else if constexpr (is_ff_v<Real>) {
      // compensated: next stage input a + f1 k as a float pair, FP64
      // accumulator a + (f1 + f2) k (or a + f1 k) from the FF increment
      const bool mid = mode == MODE_RK_MID;
#pragma unroll
      for (int fld = 0; fld < F; ++fld) {
        const size_t g = g0 + fld * N;
        const double a = sd.A[g];
        if (mid) {
          float ah, al;
          f64_split(a, ah, al);
          static_cast<FF*>(sd.Xout)[g] = FF(ah, al) + FF(sd.f1_hi, sd.f1_lo) * k[fld];
        }
        const FF inc = (mid ? FF(sd.fb_hi, sd.fb_lo) : FF(sd.f1_hi, sd.f1_lo)) * k[fld];
        sd.Aout[g] = a + (f32_to_f64(inc.hi) + f32_to_f64(inc.lo));
      }
    } else {
      // one FP64 operation per value whatever the mode (a data-independent
      // select of the coefficients, so nothing is if-converted twice)
      const bool mid = mode == MODE_RK_MID;
#pragma unroll
      for (int fld = 0; fld < F; ++fld) {
        const size_t g = g0 + fld * N;
        const double a = sd.A[g];
        if constexpr (is_f64_v<Real>) {
          const double xn = a + sd.f1 * k[fld];
          if (mid) static_cast<OutT*>(sd.Xout)[g] = static_cast<OutT>(xn);
          sd.Aout[g] = fma(mid ? sd.f2 : 0.0, k[fld], xn);
        } else {
          const float kf = k[fld];
          if (mid) static_cast<OutT*>(sd.Xout)[g] = static_cast<OutT>(fmaf(sd.f1f, kf, f64_to_f32(a)));
          const float ch = mid ? sd.fb_hi : sd.f1_hi, cl2 = mid ? sd.fb_lo : sd.f1_lo;
          sd.Aout[g] = a + f32_to_f64(fmaf(ch, kf, cl2 * kf));
        }
      }
    }
    }  // points of this thread
  }
}

// ============================================================ CK kernel
// One sweep of a 1D matrix Mtx (ROWS x COLS, COLS = input extent along DIR)
// along direction DIR over the tensors of nc cells x nf fields; input
// extents I0 x I1 x I2, compile-time, per-cell strides cs_in / cs_out.
// The CK kernel's multilevel 1-D tables (basis_table: points, weights,
// derivative, traces, and the projection and interpolation matrices of
// every level) in constant memory, one copy per compute type, filled for
// the unit's point count by set_constants.  The degree-reduction and
// interpolation sweeps read their matrix entries here at compile-time
// offsets, as constant operands of the multiply-adds.
constexpr int kCkBasisMax = 1368;  // basis_total(13)
namespace {
__constant__ float c_ckb_f[kCkBasisMax];
__constant__ double c_ckb_d[kCkBasisMax];
__constant__ FF c_ckb_ff[kCkBasisMax];
}  // namespace
template <typename Real>
__device__ __forceinline__ const Real* ck_basis_const() {
  if constexpr (is_f64_v<Real>)
    return c_ckb_d;
  else if constexpr (is_ff_v<Real>)
    return c_ckb_ff;
  else
    return c_ckb_f;
}

// The 1-D matrix at offset MOFF of the constant table (ROWS x COLS, row
// major) applied along direction DIR of every field of every cell:
// in (I0 x I1 x I2 points) -> out (ROWS points along DIR).  One thread per
// (cell, field, line): the line's COLS inputs are read once and its ROWS
// outputs summed in the order j = 0..COLS-1.
template <int DIM, typename Real, int DIR, int ROWS, int I0, int I1, int I2, int MOFF>
__device__ __forceinline__ void sweep_ct(const Real* in, int cs_in, Real* out, int cs_out, int nc, int nf) {
  constexpr int O0 = DIR == 0 ? ROWS : I0;
  constexpr int O1 = DIR == 1 ? ROWS : I1;
  constexpr int O2 = DIR == 2 ? ROWS : I2;
  constexpr int TIN = I0 * (DIM > 1 ? I1 : 1) * (DIM > 2 ? I2 : 1);
  constexpr int TOUT = O0 * (DIM > 1 ? O1 : 1) * (DIM > 2 ? O2 : 1);
  constexpr int COLS = DIR == 0 ? I0 : (DIR == 1 ? I1 : I2);
  constexpr int SIN = DIR == 0 ? 1 : (DIR == 1 ? I0 : I0 * I1);
  constexpr int SOUT = DIR == 0 ? 1 : (DIR == 1 ? O0 : O0 * O1);
  // the two other directions: a (the faster one) and b, extents and strides
  constexpr int NA = DIR == 0 ? I1 : I0;
  constexpr int NB = DIM > 2 ? (DIR == 2 ? I1 : I2) : 1;
  constexpr int SAI = DIR == 0 ? I0 : 1, SAO = DIR == 0 ? O0 : 1;
  constexpr int SBI = DIR == 2 ? I0 : I0 * I1, SBO = DIR == 2 ? O0 : O0 * O1;
  constexpr int NLN = NA * NB;
  static_assert(MOFF + ROWS * COLS <= kCkBasisMax, "matrix outside the constant table");
  const Real* Mtx = ck_basis_const<Real>() + MOFF;
  for (int task = threadIdx.x; task < nc * nf * NLN; task += blockDim.x) {
    const int cf = task / NLN;  // cell * nf + field
    const int l = task - cf * NLN;
    const int cl = cf / nf;
    const int fld = cf - cl * nf;
    const int la = l % NA, lb = l / NA;
    const Real* src = in + cl * cs_in + fld * TIN + la * SAI + lb * SBI;
    Real* dst = out + cl * cs_out + fld * TOUT + la * SAO + lb * SBO;
    Real x[COLS];
#pragma unroll
    for (int j = 0; j < COLS; ++j) x[j] = src[j * SIN];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      Real acc = Real(0);
#pragma unroll
      for (int j = 0; j < COLS; ++j) acc += Mtx[r * COLS + j] * x[j];
      dst[r * SOUT] = acc;
    }
  }
}

// The 1-D matrix at offset MOFF of the constant table (ROWS x COLS) applied
// in all DIM directions: src (COLS^DIM points) -> dst (ROWS^DIM points); t1,
// t2 scratch.  Contains barriers.
template <int DIM, typename Real, int ROWS, int COLS, int MOFF>
__device__ __forceinline__ void tensor_ct(const Real* src, int cs_src, Real* dst, int cs_dst, Real* t1,
                                          Real* t2, int cs_t, int nc, int nf) {
  if constexpr (DIM == 2) {
    sweep_ct<DIM, Real, 0, ROWS, COLS, COLS, 1, MOFF>(src, cs_src, t1, cs_t, nc, nf);
    __syncthreads();
    sweep_ct<DIM, Real, 1, ROWS, ROWS, COLS, 1, MOFF>(t1, cs_t, dst, cs_dst, nc, nf);
    __syncthreads();
  } else {
    sweep_ct<DIM, Real, 0, ROWS, COLS, COLS, COLS, MOFF>(src, cs_src, t1, cs_t, nc, nf);
    __syncthreads();
    sweep_ct<DIM, Real, 1, ROWS, ROWS, COLS, COLS, MOFF>(t1, cs_t, t2, cs_t, nc, nf);
    __syncthreads();
    sweep_ct<DIM, Real, 2, ROWS, ROWS, ROWS, COLS, MOFF>(t2, cs_t, dst, cs_dst, nc, nf);
    __syncthreads();
  }
}

// Derivative of the field set S at level with M points per direction, at
// point qq: out_u_d = rho^{-1} d_d S_p, out_p = rho c^2 div S_u
// (integrate_taylor_cauchykovalewski_step, wave_equation_operations.cc:1096-1197).
template <int DIM, int M, typename Real, bool CART>
__device__ __forceinline__ void ck_deriv(const Real* D, const Real* x, const Real* Sv,
                                         const Real* sGeo, Real rho, Real c_sq, int qq, Real* out,
                                         const Real* sJ = nullptr) {
  constexpr int NM = ipow_c(M, DIM);
  int i[3] = {0, 0, 0};
  i[0] = qq % M;
  if constexpr (DIM > 1) i[1] = (qq / M) % M;
  if constexpr (DIM > 2) i[2] = qq / (M * M);
  Real g[DIM + 1][DIM];
#pragma unroll
  for (int fld = 0; fld <= DIM; ++fld) {
#pragma unroll
    for (int e = 0; e < DIM; ++e) {
      constexpr int dummy = 0;
      (void)dummy;
      const int str = (e == 0) ? 1 : (e == 1 ? M : M * M);
      const Real* row = D + i[e] * M;
      const Real* line = Sv + fld * NM + qq - i[e] * str;
      Real s = Real(0);
#pragma unroll
      for (int a = 0; a < M; ++a) s += row[a] * line[a * str];
      g[fld][e] = s;
    }
  }
  Real xi[DIM];
#pragma unroll
  for (int e = 0; e < DIM; ++e) xi[e] = x[i[e]];
  Real JiT[DIM][DIM];
  if (sJ) {
    // cached at this point: [DIM*DIM][M^DIM] of the cell
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int e = 0; e < DIM; ++e) JiT[d][e] = sJ[(d * DIM + e) * NM + qq];
  } else {
    cell_geom<DIM, Real, CART>(sGeo, xi, JiT);
  }
  Real div = Real(0);
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int e = 0; e < DIM; ++e) div += g[d][e] * JiT[d][e];
  const Real rho_inv = Real(1) / rho;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    Real pg = Real(0);
#pragma unroll
    for (int e = 0; e < DIM; ++e) pg += g[DIM][e] * JiT[d][e];
    out[d] = rho_inv * pg;
  }
  out[DIM] = c_sq * rho * div;
}

// Accumulator of the Taylor sum: a float pair on the FP32 path, else the
// compute type (FP64 or float-float).
template <typename Real>
using CkAcc = std::conditional_t<std::is_same<Real, float>::value, FF, Real>;
template <typename Acc, typename T>
__device__ __forceinline__ void ck_acc_add(Acc& a, T v) {
  if constexpr (is_ff_v<Acc> && !is_ff_v<T>) {
    float s, e;
    two_sum(a.hi, v, s, e);
    a = FF(s, __fadd_rn(a.lo, e));
  } else {
    a += v;
  }
}
template <typename OutT, typename Acc>
__device__ __forceinline__ OutT ck_acc_out(Acc a) {
  if constexpr (is_ff_v<Acc> && !is_ff_v<OutT>)
    return static_cast<OutT>(__fadd_rn(a.hi, a.lo));
  else
    return static_cast<OutT>(a);
}

// Shared state of one CK work item.
template <typename Real>
struct CkState {
  Real* sB;
  Real* sS;
  Real* sT1;
  Real* sT2;
  Real* sm;
  const Real* sJ;  // level-0 Jacobian cache of the item (nullptr: none)
  const int* C;  // level contribution offsets (in units of Real)
  const Real* sGeo;
  int cl, q, nc;
  bool active;
  Real rho, c_sq;
};

// Recursive steps s = S..NSTEPS-1 of the Cauchy-Kovalevskaya procedure:
// derivative j = s + 2 at level r = s/2 (M = NP - 2r points per direction),
// added to the level's contribution; after odd steps the field set is
// L2-projected onto the next lower level (degree - 2).
// Without spectral evaluation (SPEC false) every step stays on level 0: in the
// Gauss collocation basis the reference's submit / integrate / inverse mass
// of each derivative (wave_equation_operations.cc:1205-1233) is the identity,
// so only the degree reduction goes away.
template <int DIM, int NP, typename Real, bool CART, int S, int NSTEPS, typename Acc, bool SPEC>
__device__ __forceinline__ void ck_steps(CkState<Real>& st, const Real* fac, Acc* c0) {
  constexpr int F = DIM + 1, N = ipow_c(NP, DIM);
  constexpr int R = SPEC ? S / 2 : 0;
  constexpr int M = NP - 2 * R;
  constexpr int NM = ipow_c(M, DIM);
  constexpr int GEO = CART ? DIM : (1 << DIM) * DIM;
  const Level<Real> L = get_level(st.sB, NP, R);
  Real sn[F];
  const bool act = st.active && st.q < NM;
  if (act)
    ck_deriv<DIM, M, Real, CART>(L.D, L.x, st.sS + st.cl * F * N, st.sGeo + st.cl * GEO, st.rho,
                                 st.c_sq, st.q, sn,
                                 (R == 0 && st.sJ) ? st.sJ + st.cl * DIM * DIM * N : nullptr);
  __syncthreads();
  if (act) {
    const Real f = fac[S];
#pragma unroll
    for (int fld = 0; fld < F; ++fld) {
      st.sS[st.cl * F * N + fld * NM + st.q] = sn[fld];
      if constexpr (R == 0)
        ck_acc_add(c0[fld], f * sn[fld]);
      else
        st.sm[st.C[R] + st.cl * F * NM + fld * NM + st.q] += f * sn[fld];
    }
  }
  __syncthreads();
  if constexpr (S + 1 < NSTEPS) {
    if constexpr (SPEC && S % 2 == 1) {
      // projection P of level R + 1 ((M - 2) x M)
      constexpr int POFF = basis_offset(NP, R + 1) + 4 * (M - 2) + (M - 2) * (M - 2);
      tensor_ct<DIM, Real, M - 2, M, POFF>(st.sS, F * N, st.sS, F * N, st.sT1, st.sT2, F * N, st.nc, F);
    }
    ck_steps<DIM, NP, Real, CART, S + 1, NSTEPS, Acc, SPEC>(st, fac, c0);
  }
}

// Bottom-up: contribution of level R interpolated to level R-1 and added.
template <int DIM, int NP, typename Real, int R, typename Acc>
__device__ __forceinline__ void ck_gather(CkState<Real>& st, Acc* c0) {
  if constexpr (R >= 1) {
    constexpr int F = DIM + 1, N = ipow_c(NP, DIM);
    constexpr int M = NP - 2 * R, MP = M + 2;
    constexpr int NMP = ipow_c(MP, DIM);
    // interpolation E of level R ((M + 2) x M)
    constexpr int EOFF = basis_offset(NP, R) + 4 * M + M * M + M * MP;
    Real* up = (DIM == 2) ? st.sT2 : st.sT1;
    tensor_ct<DIM, Real, MP, M, EOFF>(st.sm + st.C[R], F * ipow_c(M, DIM), up, F * N, st.sT1, st.sT2,
                                F * N, st.nc, F);
    if constexpr (R - 1 == 0) {
      if (st.active) {
#pragma unroll
        for (int fld = 0; fld < F; ++fld) ck_acc_add(c0[fld], up[st.cl * F * N + fld * NMP + st.q]);
      }
    } else {
      for (int idx = threadIdx.x; idx < st.nc * F * NMP; idx += blockDim.x) {
        const int c2 = idx / (F * NMP);
        const int rr = idx - c2 * F * NMP;
        st.sm[st.C[R - 1] + c2 * F * NMP + rr] += up[c2 * F * N + rr];
      }
    }
    __syncthreads();
    ck_gather<DIM, NP, Real, R - 1, Acc>(st, c0);
  }
}

// Real-sized words per stored input value (staging area of the CK kernel)
template <typename Real, typename InT>
constexpr int ck_in_words() {
  return (int)((sizeof(InT) + sizeof(Real) - 1) / sizeof(Real));
}

template <int DIM, int NP, typename Real, typename InT, typename OutT, bool CART, bool POST,
          bool SPEC = true>
__global__ void __maxnreg__(sizeof(Real) == 8 ? 128 : 80) ck_kernel(const LaunchArgs La) {
  using S = Shape<DIM, NP, CART>;
  constexpr int F = S::F, N = S::N;
  constexpr int NL = n_levels(NP);
  // Taylor terms j = 0..max(k,2); derivatives j >= 2 come from the steps
  constexpr int NSTEPS = (NP - 2 > 1) ? NP - 2 : 1;
  constexpr int RLAST = SPEC ? (NSTEPS - 1) / 2 : 0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sm = reinterpret_cast<Real*>(smem_raw);
  const int CB = La.cells_per_block;
  const CkSmem<DIM, NP, CART> lay(CB, ck_in_words<Real, InT>());
  Real* sB = sm + lay.op.basis;
  Real* sX = sm + lay.op.X;
  Real* sG = sm + lay.op.G;
  Real* sFl = sm + lay.op.Fl;
  Real* sGeo = sm + lay.op.geo;
  Real* sMat = sm + lay.op.mat;
  if ((int)blockDim.x != CB * N) {
    if (threadIdx.x == 0) atomicOr(La.err, ERR_BAD_LAUNCH);
    return;
  }
  load_basis<Real>(La.basis, sB, basis_total(NP));
  Real fac[12];
#pragma unroll
  for (int s = 0; s < 12; ++s) {
    if constexpr (is_f64_v<Real>)
      fac[s] = La.ck_fac_d[s];
    else if constexpr (is_ff_v<Real>)
      fac[s] = FF::from_double(La.ck_fac_d[s]);
    else
      fac[s] = La.ck_fac[s];
  }
  Real dtr, half_dt2;
  if constexpr (is_f64_v<Real>) {
    dtr = La.ck_dt_d;
    half_dt2 = La.ck_half_dt2_d;
  } else if constexpr (is_ff_v<Real>) {
    dtr = FF::from_double(La.ck_dt_d);
    half_dt2 = FF::from_double(La.ck_half_dt2_d);
  } else {
    dtr = La.ck_dt;
    half_dt2 = La.ck_half_dt2;
  }

  // Work items are pipelined: the next item's inputs, geometry and
  // materials are copied asynchronously (cp.async, one value per copy) into
  // the staging area while the current item is computed, and converted into
  // the compute layout when its turn comes.
  const InT* sPX = reinterpret_cast<const InT*>(sm + lay.P);
  auto prefetch = [&](int wn) {
    const WorkItem wj = La.work[wn];
    const SolveDesc sdn = pick(La, wj.solve);
    const int tot = wj.n_cells * F * N;
    const InT* X = static_cast<const InT*>(sdn.X) + (size_t)wj.cell_begin * F * N;
    InT* px = reinterpret_cast<InT*>(sm + lay.P);
    for (int i = threadIdx.x; i < tot; i += blockDim.x) cp_async<sizeof(InT)>(px + i, X + i);
    const Real* G = static_cast<const Real*>(sdn.geo) + (size_t)wj.cell_begin * S::GEO;
    for (int i = threadIdx.x; i < wj.n_cells * S::GEO; i += blockDim.x)
      cp_async<sizeof(Real)>(sm + lay.PG + i, G + i);
    const Real* M = static_cast<const Real*>(sdn.mat) + (size_t)wj.cell_begin * 4;
    for (int i = threadIdx.x; i < wj.n_cells * 4; i += blockDim.x) cp_async<sizeof(Real)>(sm + lay.PM + i, M + i);
    cp_async_commit();
  };
  if ((int)blockIdx.x < La.n_work) prefetch(blockIdx.x);

  for (int w = blockIdx.x; w < La.n_work; w += gridDim.x) {
    const WorkItem wi = La.work[w];
    const SolveDesc sd = pick(La, wi.solve);
    const int nc = wi.n_cells;
    cp_async_wait_all();
    // the previous item is done with the compute layout; this item's staged
    // values (every thread's copies) are visible
    __syncthreads();
    for (int i = threadIdx.x; i < nc * F * N; i += blockDim.x) sX[i] = to_real<Real>(sPX[i]);
    for (int i = threadIdx.x; i < nc * S::GEO; i += blockDim.x) sGeo[i] = sm[lay.PG + i];
    for (int i = threadIdx.x; i < nc * 4; i += blockDim.x) sMat[i] = sm[lay.PM + i];
    for (int r = 1; r < NL; ++r) {
      const int sz = nc * F * ipow_rt(NP - 2 * r, DIM);
      for (int i = threadIdx.x; i < sz; i += blockDim.x) sm[lay.C[r] + i] = Real(0);
    }
    __syncthreads();
    const int cl = threadIdx.x / N;
    const int q = threadIdx.x - cl * N;
    const bool active = cl < nc;
    const Real rho = active ? sMat[4 * cl] : Real(1);
    const Real cc = active ? sMat[4 * cl + 1] : Real(1);
    const Real c_sq = cc * cc;
    // inverse-transpose Jacobian at this thread's level-0 point, evaluated
    // once and read back (by this thread only) by every level-0 derivative
    Real* sJ = CART ? nullptr : sm + lay.J;
    if constexpr (!CART) {
      if (active) {
        const Level<Real> L0 = get_level(sB, NP, 0);
        int i[3] = {0, 0, 0};
        split_point<DIM, NP>(q, i);
        Real xi[DIM];
#pragma unroll
        for (int e = 0; e < DIM; ++e) xi[e] = L0.x[i[e]];
        Real JiT[DIM][DIM];
        cell_geom<DIM, Real, false>(sGeo + cl * S::GEO, xi, JiT);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
#pragma unroll
          for (int e = 0; e < DIM; ++e) sJ[(cl * DIM * DIM + d * DIM + e) * N + q] = JiT[d][e];
      }
    }
    Real d1[F];
    if constexpr (POST) {
      // first time derivative = full DG operator (recongraddiv = apply(src))
      Real Ru[DIM];
      Real inv_jxw = Real(1);
      if (active) op_cell<DIM, NP, Real, CART>(sB, sX, sG, sGeo, sMat, cl, q, Real(1), Ru, inv_jxw);
      for (int fp = threadIdx.x; fp < nc * 2 * DIM * S::NF; fp += blockDim.x)
        op_face<DIM, NP, Real, InT, CART>(sB, sX, sFl, sGeo, sMat, sd, wi.cell_begin, nc, fp,
                                          Real(1), La.err);
      __syncthreads();
      if (active) op_collect<DIM, NP, Real, CART>(sB, sG, sFl, cl, q, Ru, inv_jxw, d1);
    } else {
      if (active) {
        Real o[F];
        const Level<Real> L0 = get_level(sB, NP, 0);
        ck_deriv<DIM, NP, Real, CART>(L0.D, L0.x, sX + cl * F * N, sGeo + cl * S::GEO, rho, c_sq,
                                      q, o, CART ? nullptr : sJ + cl * DIM * DIM * N);
#pragma unroll
        for (int fld = 0; fld < F; ++fld) d1[fld] = -o[fld];
      }
    }
    // Taylor terms 0 and 1; the recursion starts from S = -du/dt.  The
    // Taylor sum is accumulated in the compute type, except on the FP32
    // path, where it is a float pair: term 0 is dt * u from the FP64 state
    // (both split exactly into pairs), and every later term is added with an
    // error-free two-sum, so that the sum carries about 44 bits like the
    // FP64 state it is added to; it is rounded once, to the FP32 stage input
    // T of the second step.
    Real* sS = sm + lay.Sv;
    using Acc = CkAcc<Real>;
    Acc c0[F];
    if (active) {
#pragma unroll
      for (int fld = 0; fld < F; ++fld) {
        if constexpr (is_ff_v<Acc> && !is_ff_v<Real>) {
          float uh, ul;
          if constexpr (is_f64_v<InT>) {
            f64_split(sPX[cl * F * N + fld * N + q], uh, ul);
          } else {
            uh = sX[cl * F * N + fld * N + q];
            ul = 0.f;
          }
          c0[fld] = FF::from_double(La.ck_dt_d) * FF(uh, ul);
          ck_acc_add(c0[fld], half_dt2 * d1[fld]);
        } else {
          c0[fld] = dtr * sX[cl * F * N + fld * N + q] + half_dt2 * d1[fld];
        }
        sS[cl * F * N + fld * N + q] = -d1[fld];
      }
    }
    __syncthreads();
    // every read of the staging area is done: the next item may land there
    if (w + (int)gridDim.x < La.n_work) prefetch(w + gridDim.x);
    CkState<Real> st;
    st.sB = sB;
    st.sS = sS;
    st.sT1 = sm + lay.T1;
    st.sT2 = sm + lay.T2;
    st.sm = sm;
    st.sJ = sJ;
    st.C = lay.C;
    st.sGeo = sGeo;
    st.cl = cl;
    st.q = q;
    st.nc = nc;
    st.active = active;
    st.rho = rho;
    st.c_sq = c_sq;
    ck_steps<DIM, NP, Real, CART, 0, NSTEPS, Acc, SPEC>(st, fac, c0);
    ck_gather<DIM, NP, Real, RLAST, Acc>(st, c0);
    if (active) {
      OutT* T = static_cast<OutT*>(sd.Xout);
      const size_t g0 = ((size_t)wi.cell_begin + cl) * F * N + q;
#pragma unroll
      for (int fld = 0; fld < F; ++fld) T[g0 + fld * N] = ck_acc_out<OutT>(c0[fld]);
    }
  }
}

}  // namespace ew
