// ew_cart.cuh -- stage kernel for Cartesian (axis-aligned box) cells.
//
// On a Cartesian cell the Jacobian is diag(h), so in direction e only the
// velocity component u_e and the pressure interact: the cell term gives
// k_{u_e} = -rho^{-1}/h_e d_e p and a pressure part rho c^2/h_e (D^T w u_e)/w,
// and the faces normal to e lift only u_e and p.  The kernel therefore runs
// one thread per (cell, direction, line): it holds the line of u_e and p in
// registers, evaluates both face traces, the neighbours' traces, the two
// upwind fluxes, the derivative and weighted-transpose contractions with
// even-odd splitting (half the multiply-adds), and finishes the update of
// u_e on that line; pressure contributions of the directions meet in shared
// memory and are finished by one thread per point.
//
// Input staging: each work item's contiguous block of cells (stage input X
// and accumulator A) is copied into shared memory with one 1-D bulk copy
// (cp.async.bulk, TMA engine) per array, completed on an mbarrier.  The
// copy of the next item's X is issued before the current one is processed
// (double buffering); A, read only by the epilogue, has a single buffer
// refilled at the start of each item, which keeps the block small enough
// for four resident blocks per SM.  Waits are bounded; on time-out the
// kernel raises ERR_WAIT_TIMEOUT and stops.
//
// Compute types: FP64 (the reference's arithmetic), FP32 (mixed precision)
// or FF, an unevaluated float pair (ew_ff.cuh) for the compensated
// precision: stage inputs, constants and every sum and product of the line
// work in float-float, about 44 significant bits on the FP32 pipes.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "ew_ff.cuh"
#include "ew_kernels.cuh"

namespace ew {

constexpr int ERR_WAIT_TIMEOUT = 8;

// acc + a * b in a chain of sums, and the end of the chain (float-float:
// fused, with one renormalisation at the end; FP32 / FP64: a fused multiply-add)
template <typename R>
__device__ __forceinline__ R mac(R acc, R a, R b) {
  if constexpr (std::is_same<R, FF>::value)
    return ff_mac(acc, a, b);
  else
    return acc + a * b;
}
template <typename R>
__device__ __forceinline__ R end_sum(R v) {
  if constexpr (std::is_same<R, FF>::value)
    return ff_norm(v);
  else
    return v;
}

// Even-odd form of an NP x NP matrix M with M[n-1-i][n-1-j] = -M[i][j]:
// for i < H = NP/2, a_i = sum_j P_ij e_j (+ mid_col_i x_m), b_i = sum_j Q_ij o_j,
// y_i = a_i + b_i, y_{n-1-i} = b_i - a_i, and for odd NP y_m = sum_j mid_row_j o_j,
// with e_j = x_j + x_{n-1-j}, o_j = x_j - x_{n-1-j}.
// Sizes for up to 13 points per line (degree 12): H = NP / 2 <= 6.
constexpr int kEoMax = 6;
constexpr int kLineMax = 16;

template <typename Real>
struct EoMat {
  Real P[kEoMax][kEoMax], Q[kEoMax][kEoMax];
  Real mid_row[kEoMax], mid_col[kEoMax];
};

template <typename Real>
struct CartBasis {
  EoMat<Real> D;   // D[i][j] = l_j'(x_i)
  EoMat<Real> Dt;  // Dt[i][a] = D[a][i] w_a / w_i
  Real Ls[kEoMax], La[kEoMax], Lmid;  // traces: t0 = s + a, t1 = s - a
  Real Ws[kEoMax], Wa[kEoMax], Wmid;  // lifts with l_j(s)/w_j
  Real L[2][kLineMax];                // l_j(0), l_j(1) (neighbour traces)
};

// Host-side construction from the 1D Gauss data.
inline void make_eo(const double* M, int NP, EoMat<double>& E) {
  const int H = NP / 2;
  for (int i = 0; i < kEoMax; ++i)
    for (int j = 0; j < kEoMax; ++j) E.P[i][j] = E.Q[i][j] = 0.0;
  for (int i = 0; i < kEoMax; ++i) E.mid_row[i] = E.mid_col[i] = 0.0;
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < H; ++j) {
      E.P[i][j] = 0.5 * (M[i * NP + j] + M[i * NP + NP - 1 - j]);
      E.Q[i][j] = 0.5 * (M[i * NP + j] - M[i * NP + NP - 1 - j]);
    }
  if (NP % 2) {
    const int m = NP / 2;
    for (int j = 0; j < H; ++j) E.mid_row[j] = M[m * NP + j];
    for (int i = 0; i < H; ++i) E.mid_col[i] = M[i * NP + m];
  }
}

template <int NP, typename Real>
__device__ __forceinline__ void eo_apply(const EoMat<Real>& M, const Real* e, const Real* o,
                                         Real xm, Real* a, Real* b) {
  constexpr int H = NP / 2;
#pragma unroll
  for (int i = 0; i < H; ++i) {
    Real s = Real(0), t = Real(0);
#pragma unroll
    for (int j = 0; j < H; ++j) {
      s = mac(s, M.P[i][j], e[j]);
      t = mac(t, M.Q[i][j], o[j]);
    }
    if constexpr (NP % 2 == 1) s = mac(s, M.mid_col[i], xm);
    a[i] = end_sum(s);
    b[i] = end_sum(t);
  }
  if constexpr (NP % 2 == 1) {
    Real s = Real(0);
#pragma unroll
    for (int j = 0; j < H; ++j) s = mac(s, M.mid_row[j], o[j]);
    a[H] = end_sum(s);  // middle output (no pair)
  }
}

// One copy per instantiation unit (each unit serves one NP); filled from
// the host by set_cart_constants for the current device.
namespace {
__constant__ CartBasis<float> c_cart_f;
__constant__ CartBasis<double> c_cart_d;
__constant__ CartBasis<FF> c_cart_ff;
}  // namespace
template <typename Real>
struct CartConst;
template <>
struct CartConst<float> {
  static __device__ __forceinline__ const CartBasis<float>& get() { return c_cart_f; }
};
template <>
struct CartConst<double> {
  static __device__ __forceinline__ const CartBasis<double>& get() { return c_cart_d; }
};
template <>
struct CartConst<FF> {
  static __device__ __forceinline__ const CartBasis<FF>& get() { return c_cart_ff; }
};

// Magnitudes of the 1-D coefficients (their float parts) for the compensated
// kernel: every anchored line sum (ew_ff.cuh) takes its anchor from
// sum_j |c_j| |x_j| of its own terms, computed with these.
struct FfBounds {
  float aDP[kEoMax][kEoMax], aDQ[kEoMax][kEoMax], aDmc[kEoMax], aDmr[kEoMax];
  float aTP[kEoMax][kEoMax], aTQ[kEoMax][kEoMax], aTmc[kEoMax], aTmr[kEoMax];
  float aWs[kEoMax], aWa[kEoMax], aWmid;
  float aLs[kEoMax], aLa[kEoMax], aLmid, aL[2][kLineMax];
};
namespace {
__constant__ FfBounds c_ff_bounds;
}  // namespace

// Host: even-odd constants from the 1D Gauss data of NP points.
inline CartBasis<double> make_cart_basis(int NP, const double* w, const double* D,
                                         const double* L0, const double* L1) {
  CartBasis<double> c;
  std::memset(&c, 0, sizeof(c));
  make_eo(D, NP, c.D);
  double Dt[kLineMax * kLineMax];
  for (int i = 0; i < NP; ++i)
    for (int a = 0; a < NP; ++a) Dt[i * NP + a] = D[a * NP + i] * w[a] / w[i];
  make_eo(Dt, NP, c.Dt);
  const int H = NP / 2;
  for (int j = 0; j < H; ++j) {
    c.Ls[j] = 0.5 * (L0[j] + L0[NP - 1 - j]);
    c.La[j] = 0.5 * (L0[j] - L0[NP - 1 - j]);
    const double a = L0[j] / w[j], b = L0[NP - 1 - j] / w[NP - 1 - j];
    c.Ws[j] = 0.5 * (a + b);
    c.Wa[j] = 0.5 * (a - b);
  }
  if (NP % 2) {
    c.Lmid = L0[NP / 2];
    c.Wmid = L0[NP / 2] / w[NP / 2];
  }
  for (int j = 0; j < NP; ++j) {
    c.L[0][j] = L0[j];
    c.L[1][j] = L1[j];
  }
  return c;
}

inline FfBounds make_ff_bounds(const CartBasis<double>& c) {
  FfBounds f;
  for (int i = 0; i < kEoMax; ++i) {
    for (int j = 0; j < kEoMax; ++j) {
      f.aDP[i][j] = std::fabs((float)c.D.P[i][j]);
      f.aDQ[i][j] = std::fabs((float)c.D.Q[i][j]);
      f.aTP[i][j] = std::fabs((float)c.Dt.P[i][j]);
      f.aTQ[i][j] = std::fabs((float)c.Dt.Q[i][j]);
    }
    f.aDmc[i] = std::fabs((float)c.D.mid_col[i]);
    f.aDmr[i] = std::fabs((float)c.D.mid_row[i]);
    f.aTmc[i] = std::fabs((float)c.Dt.mid_col[i]);
    f.aTmr[i] = std::fabs((float)c.Dt.mid_row[i]);
    f.aWs[i] = std::fabs((float)c.Ws[i]);
    f.aWa[i] = std::fabs((float)c.Wa[i]);
  }
  f.aWmid = std::fabs((float)c.Wmid);
  for (int j = 0; j < kEoMax; ++j) {
    f.aLs[j] = std::fabs((float)c.Ls[j]);
    f.aLa[j] = std::fabs((float)c.La[j]);
  }
  f.aLmid = std::fabs((float)c.Lmid);
  for (int j = 0; j < kLineMax; ++j) {
    f.aL[0][j] = std::fabs((float)c.L[0][j]);
    f.aL[1][j] = std::fabs((float)c.L[1][j]);
  }
  return f;
}

template <typename Real>
inline CartBasis<Real> cast_basis(const CartBasis<double>& d) {
  CartBasis<Real> r;
  const double* src = reinterpret_cast<const double*>(&d);
  Real* dst = reinterpret_cast<Real*>(&r);
  for (size_t i = 0; i < sizeof(d) / sizeof(double); ++i) {
    if constexpr (is_ff_v<Real>)
      dst[i] = FF::from_double(src[i]);  // each constant as float + float remainder
    else
      dst[i] = static_cast<Real>(src[i]);
  }
  return r;
}

// ---------------------------------------------------------------- mbarrier / bulk copy

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// transaction bytes announced without an arrival, and an arrival alone
__device__ __forceinline__ void mbar_add_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Bounded wait for the phase with the given parity; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = (1 << 22)) {
  const uint32_t a = smem_addr(bar);
  for (int it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Per-cell constants kept in shared memory: rho^{-1}, rho c^2, tau = 1/(c rho),
// 1/tau, 1/h_e (3), and per face (tau of the neighbour, 1/(tau + tau_nb)).
constexpr int kCellConsts = 4 + 3 + 6 * 2;

// Shared-memory layout of the Cartesian kernel (bytes); AB is the size of
// one staged accumulator element (8: FP64 or float pair, 4: the lo part).
// Neighbour field arrays by bulk copy (else per-thread line copies): 3-D
// with at least 6 points per line, and with 4 for FP32 stage inputs.
// Measured per LSRK45 step (about 226 M DoFs): mixed k = 3 / 5 / 6 / 7 gain
// 1 / 6 / 8 / 6 %, k = 4 loses 4 % (more registers for the window offsets)
// and k = 2 loses 37 % (108-byte arrays: the copies' fixed cost dominates);
// the compensated k = 3 kernel (8-byte inputs) lost 16 %.
template <int DIM, int NP, typename InT>
__host__ __device__ constexpr bool cart_nb_bulk() {
  return DIM == 3 && (NP >= 6 || (NP == 4 && sizeof(InT) == 4));
}

template <int DIM, int NP, typename Real, typename InT, int AB = 8>
struct CartSmem {
  static constexpr int N = ipow_c(NP, DIM);
  static constexpr int F = DIM + 1;
  // one field array of a neighbour copied in bulk: the array rounded out to
  // 16-byte boundaries at both ends (exactly the array when its size and
  // start are multiples of 16)
  static constexpr int NB_SLOT = (N * sizeof(InT)) % 16 == 0
                                     ? (int)(N * sizeof(InT))
                                     : (int)(((N * sizeof(InT) + 15) & ~(size_t)15) + 16);
  size_t bar, X, A, Kp, cell, nb, end;
  int xbytes, abytes;  // per buffer
  // The stage input X is double buffered (the next item's copy is in
  // flight while the current one is processed).  The accumulator A is only
  // read by the epilogue: when X is staged on its own, A has one buffer,
  // refilled at the start of every item; when X == A (first stage), A is
  // the operator input and is double buffered like X.
  __host__ __device__ static bool a_single(bool stage_x, bool stage_a) { return stage_a && stage_x; }
  __host__ __device__ CartSmem(int CB, bool stage_x, bool stage_a) {
    bar = 0;  // mbarriers: X / A double buffered (0, 1), single A (2)
    X = 64;
    xbytes = stage_x ? CB * F * N * (int)sizeof(InT) : 0;
    A = X + 2 * (size_t)((xbytes + 127) & ~127);
    abytes = stage_a ? CB * F * N * AB : 0;
    Kp = A + (a_single(stage_x, stage_a) ? 1 : 2) * (size_t)((abytes + 127) & ~127);
    cell = Kp + (size_t)DIM * CB * N * sizeof(Real);
    // per thread: the neighbours' lines of u_e and p on both sides; or, with
    // bulk copies, per (cell, face) the neighbour's u_e and p arrays in
    // slots of NB_SLOT bytes
    nb = (cell + (size_t)CB * kCellConsts * sizeof(Real) + 15) & ~(size_t)15;
    const int threads = CB * DIM * ipow_c(NP, DIM - 1);
    const size_t lines = (size_t)threads * 4 * NP * sizeof(InT);
    const size_t slots = cart_nb_bulk<DIM, NP, InT>() ? (size_t)CB * 2 * DIM * 2 * NB_SLOT : 0;
    end = nb + (lines > slots ? lines : slots);
    end = (end + 127) & ~(size_t)127;
  }
};

// Epilogues of the stage kernel (compile-time, so that no FP64 work of
// an unused branch is if-converted into the executed path).
//  APPLY       : Aout = k (WaveEquationOperation::apply)
//  F64_MID/LAST: the reference's RKVectorUpdater arithmetic in FP64
//  MIX_S1      : first LSRK stage, FP64 state in (split into float pairs
//                in shared memory), FP32 stage input and float-float
//                accumulator out
//  MIX_MID     : float-float accumulator in and out, FP32 stage input out
//  MIX_LAST    : float-float accumulator in, FP64 state out
//  MIX_UPD     : FP64 in, FP64 out (ADER update u + k)
//  MIX_S1_FF   : first stage of a step inside a multi-step call: the state
//                is a float pair held as two FP32 arrays, hi (the stage
//                input X, read like a middle stage's) and lo (staged in
//                place of A)
//  MIX_LAST_FF : last stage of such a step: the new state is left as that
//                pair, hi to Xout and lo to Aout (no rounding to FP64)
//  FF_LAST_PAIR: compensated operator, last stage of a step inside a
//                multi-step call: the new state is written as float pairs
//                (8 bytes, like the FP64 value it stands for) to Aout; the
//                next step's first stage reads it like a middle stage reads
//                its input and accumulator (X == A)
// Within an LSRK step the mixed path keeps the accumulator as an unevaluated
// sum hi + lo of two floats (about 48 significant bits) in the 8-byte slot
// of the FP64 vector, updated with error-free transformations on the FP32
// pipes; the FP64 pipe is used only where the step begins and ends.
enum Epi : int {
  EPI_APPLY = 0,
  EPI_F64_MID = 1,
  EPI_F64_LAST = 2,
  EPI_MIX_S1 = 3,
  EPI_MIX_MID = 4,
  EPI_MIX_LAST = 5,
  EPI_MIX_UPD = 6,
  EPI_MIX_S1_FF = 7,
  EPI_MIX_LAST_FF = 8,
  EPI_FF_LAST_PAIR = 9
};

template <int EPI>
struct EpiTraits {
  static constexpr bool stage_a = EPI != EPI_APPLY;
  static constexpr bool writes_x = EPI == EPI_F64_MID || EPI == EPI_MIX_S1 || EPI == EPI_MIX_MID ||
                                   EPI == EPI_MIX_S1_FF || EPI == EPI_MIX_LAST_FF;
  // A is the FP32 lo array of a float-pair state whose hi array is X
  static constexpr bool lo_in = EPI == EPI_MIX_S1_FF;
  // the new state is written as hi (Xout) and lo (Aout, FP32) arrays
  static constexpr bool lo_out = EPI == EPI_MIX_LAST_FF;
  static constexpr int a_elem = lo_in ? 4 : 8;
};

// (hi, lo) + b with hi + lo normalised (Knuth two-sum, fast renormalisation)
__device__ __forceinline__ void ff_add(float hi, float lo, float b, float& rh, float& rl) {
  const float s = __fadd_rn(hi, b);
  const float v = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, v)), __fsub_rn(b, v));
  const float t = __fadd_rn(e, lo);
  rh = __fadd_rn(s, t);
  rl = __fsub_rn(t, __fsub_rn(rh, s));
}

__device__ __forceinline__ double ff_pack(float hi, float lo) {
  return __hiloint2double(__float_as_int(lo), __float_as_int(hi));
}
__device__ __forceinline__ float ff_hi(double d) { return __int_as_float(__double2loint(d)); }
__device__ __forceinline__ float ff_lo(double d) { return __int_as_float(__double2hiint(d)); }

template <typename Real>
__device__ __forceinline__ double real_to_f64(Real k) {
  if constexpr (is_f64_v<Real>)
    return k;
  else if constexpr (is_ff_v<Real>)
    return f32_to_f64(k.hi) + f32_to_f64(k.lo);
  else
    return f32_to_f64(k);
}

// One value: `a` is the accumulator slot (FP64 or float-float), k the
// operator value; returns the next stage input (xn) and the new slot (an).
template <int EPI, typename Real, typename OutT>
__device__ __forceinline__ void epi_value(const SolveDesc& sd, double a, Real k, OutT& xn,
                                          double& an) {
  xn = OutT(0);
  if constexpr (is_ff_v<Real>) {
    // compensated operator: the update of the float-pair accumulator in FF
    // arithmetic too (the mixed path rounds the increment to FP32)
    static_assert(EPI == EPI_APPLY || EPI == EPI_MIX_S1 || EPI == EPI_MIX_MID || EPI == EPI_MIX_LAST ||
                      EPI == EPI_MIX_UPD || EPI == EPI_FF_LAST_PAIR,
                  "FF epilogues: apply, LSRK stages 1, middle and 5, ADER update");
    if constexpr (EPI == EPI_APPLY) {
      an = real_to_f64<Real>(k);
    } else if constexpr (EPI == EPI_MIX_UPD) {
      // ADER update u + M^-1 A(T): the FF increment rounded once to FP64
      const FF inc = FF(sd.f1_hi, sd.f1_lo) * k;
      an = a + (f32_to_f64(inc.hi) + f32_to_f64(inc.lo));
    } else if constexpr (EPI == EPI_MIX_LAST) {
      const FF r = FF(ff_hi(a), ff_lo(a)) + FF(sd.f1_hi, sd.f1_lo) * k;
      an = f32_to_f64(r.hi) + f32_to_f64(r.lo);
    } else if constexpr (EPI == EPI_FF_LAST_PAIR) {
      const FF r = FF(ff_hi(a), ff_lo(a)) + FF(sd.f1_hi, sd.f1_lo) * k;
      an = ff_pack(r.hi, r.lo);
    } else {
      const FF acc(ff_hi(a), ff_lo(a));
      xn = acc + FF(sd.f1_hi, sd.f1_lo) * k;
      const FF r = acc + FF(sd.fb_hi, sd.fb_lo) * k;
      an = ff_pack(r.hi, r.lo);
    }
  } else if constexpr (EPI == EPI_APPLY) {
    an = real_to_f64<Real>(k);
  } else if constexpr (EPI == EPI_F64_MID) {
    const double x = a + sd.f1 * k;
    xn = static_cast<OutT>(x);
    an = x + sd.f2 * k;
  } else if constexpr (EPI == EPI_F64_LAST) {
    an = a + sd.f1 * k;
  } else if constexpr (EPI == EPI_MIX_MID || EPI == EPI_MIX_S1 || EPI == EPI_MIX_S1_FF) {
    // MIX_S1: the staged FP64 state was split into (hi, lo) in place
    const float ah = ff_hi(a), al = ff_lo(a);
    xn = static_cast<OutT>(fmaf(sd.f1f, k, ah));
    float rh, rl;
    ff_add(ah, al, fmaf(sd.fb_hi, k, sd.fb_lo * k), rh, rl);
    an = ff_pack(rh, rl);
  } else if constexpr (EPI == EPI_MIX_LAST) {
    float rh, rl;
    ff_add(ff_hi(a), ff_lo(a), fmaf(sd.f1_hi, k, sd.f1_lo * k), rh, rl);
    an = f32_to_f64(rh) + f32_to_f64(rl);
  } else if constexpr (EPI == EPI_MIX_LAST_FF) {
    float rh, rl;
    ff_add(ff_hi(a), ff_lo(a), fmaf(sd.f1_hi, k, sd.f1_lo * k), rh, rl);
    xn = static_cast<OutT>(rh);
    an = ff_pack(rh, rl);
  } else {  // EPI_MIX_UPD
    an = a + f32_to_f64(fmaf(sd.f1_hi, k, sd.f1_lo * k));
  }
}

__device__ __forceinline__ void store2(float* p, float a, float b) {
  *reinterpret_cast<float2*>(p) = make_float2(a, b);
}
__device__ __forceinline__ void store2(double* p, double a, double b) {
  *reinterpret_cast<double2*>(p) = make_double2(a, b);
}
__device__ __forceinline__ void store2(FF* p, FF a, FF b) {
  *reinterpret_cast<float4*>(p) = make_float4(a.hi, a.lo, b.hi, b.lo);
}

struct CartArgs {
  LaunchArgs la;
  int32_t stage_x;   // X staged in shared memory (else read from A's buffer: X == A)
  int32_t tma;       // bulk copies usable (alignment checked on the host)
  int32_t nb_lines;  // neighbour lines by per-thread copies even where bulk copies are built
  int32_t pad;
};

#ifndef EW_FF_MAXNREG
#define EW_FF_MAXNREG 128
#endif
template <int DIM, int NP, typename Real, typename InT, int EPI>
__global__ void __maxnreg__(is_f64_v<Real> ? 96 : (is_ff_v<Real> ? EW_FF_MAXNREG : ((NP >= 7 || sizeof(InT) == 8) ? 80 : 72)))
    stage_cart_kernel(const CartArgs ca) {
  // next stage input: FP64, float pairs (compensated) or FP32
  using OutT = std::conditional_t<is_f64_v<Real>, double, std::conditional_t<is_ff_v<Real>, FF, float>>;
  constexpr bool stage_a = EpiTraits<EPI>::stage_a;
  constexpr int N = ipow_c(NP, DIM);
  constexpr int F = DIM + 1;
  constexpr int NL = ipow_c(NP, DIM - 1);
  constexpr int H = NP / 2;
  constexpr int HA = H > 0 ? H : 1;  // array extent of the even-odd halves
  constexpr bool CONV = !is_f64_v<Real> && is_f64_v<InT>;
  constexpr bool LO_IN = EpiTraits<EPI>::lo_in;
  constexpr bool LO_OUT = EpiTraits<EPI>::lo_out;
  constexpr int A_ELEM = EpiTraits<EPI>::a_elem;
  const LaunchArgs& La = ca.la;
  const int CB = La.cells_per_block;
  extern __shared__ __align__(128) unsigned char smem_cart[];
  const CartSmem<DIM, NP, Real, InT, A_ELEM> lay(CB, ca.stage_x != 0, stage_a);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_cart + lay.bar);
  const size_t xstride = (size_t)((lay.xbytes + 127) & ~127);
  const size_t astride = (size_t)((lay.abytes + 127) & ~127);
  Real* sKp = reinterpret_cast<Real*>(smem_cart + lay.Kp);
  Real* sCell = reinterpret_cast<Real*>(smem_cart + lay.cell);
  if ((int)blockDim.x != CB * DIM * NL) {
    if (threadIdx.x == 0) atomicOr(La.err, ERR_BAD_LAUNCH);
    return;
  }
  const CartBasis<Real>& B = CartConst<Real>::get();
  const bool stage_x = (sizeof(InT) == 4) || ca.stage_x != 0;

  const bool a_single = CartSmem<DIM, NP, Real, InT, A_ELEM>::a_single(stage_x, stage_a);
  // issue the copies of work item w into buffer b (X, and A unless it has
  // its own single buffer)
  auto issue = [&](const WorkItem& wi, int b) {
    const SolveDesc* sdp = La.solves ? La.solves + wi.solve : &La.single;
    const void* Xg = sdp->X;
    const size_t c0 = (size_t)wi.cell_begin * F * N;
    const char* Ag = reinterpret_cast<const char*>(sdp->A) + c0 * A_ELEM;
    const uint32_t nx = (uint32_t)(wi.n_cells * F * N * sizeof(InT));
    const uint32_t na = (uint32_t)(wi.n_cells * F * N * A_ELEM);
    uint32_t tx = 0;
    if (stage_x) tx += nx;
    if (stage_a && !a_single) tx += na;
    mbar_expect_tx(&bars[b], tx);
    if (stage_x) bulk_g2s(smem_cart + lay.X + b * xstride, static_cast<const InT*>(Xg) + c0, nx, &bars[b]);
    if (stage_a && !a_single) bulk_g2s(smem_cart + lay.A + b * astride, Ag, na, &bars[b]);
  };
  // the single A buffer of work item w
  auto issue_a = [&](const WorkItem& wi) {
    const SolveDesc* sdp = La.solves ? La.solves + wi.solve : &La.single;
    const uint32_t na = (uint32_t)(wi.n_cells * F * N * A_ELEM);
    mbar_expect_tx(&bars[2], na);
    bulk_g2s(smem_cart + lay.A, reinterpret_cast<const char*>(sdp->A) + (size_t)wi.cell_begin * F * N * A_ELEM,
             na, &bars[2]);
  };

  // line task of this thread: (cell, direction, line), the same for every item
  const int tcl = threadIdx.x / (DIM * NL);
  const int te = (threadIdx.x - tcl * DIM * NL) / NL;
  const int tt = threadIdx.x - tcl * DIM * NL - te * NL;
  int tbase = 0;
  {
    int ti[3] = {0, 0, 0};
    tbase = face_base<DIM, NP>(te, tt, ti);
  }
  const int tstr = dir_stride(te, NP);
  // slot element k of this thread at k * blockDim.x + threadIdx.x (conflict-free)
  InT* nslot = reinterpret_cast<InT*>(smem_cart + lay.nb) + threadIdx.x;
  const int nstride = blockDim.x;
  // With bulk copies usable, the same area holds whole neighbour field
  // arrays instead: slot (cell * 2 DIM + face) * 2 + (u_e, p), each filled by
  // one bulk copy of the array rounded out to 16-byte boundaries, completed
  // on bars[3].  Bulk copies are enabled only when a
  // cell's data is a multiple of 16 bytes, so that the rounded windows stay
  // inside the stage input array.
  constexpr int NB_SLOT = CartSmem<DIM, NP, Real, InT, A_ELEM>::NB_SLOT;
  const bool nb_bulk = cart_nb_bulk<DIM, NP, InT>() && ca.tma != 0 && ca.nb_lines == 0;
  unsigned char* sNb = smem_cart + lay.nb;
  // byte offset of a neighbour's field array within its 16-byte window
  auto nb_rem = [](int nb, int f) -> int {
    return (int)((((size_t)nb * F + f) * N * sizeof(InT)) & 15);
  };
  // the neighbours of this thread's line (both sides); boundary: -id
  auto lookup_nb = [&](const WorkItem& wi, const SolveDesc& sd, int* nbs) {
    nbs[0] = nbs[1] = -EW_BC_HARD_WALL_ID;
    if (tcl < wi.n_cells) {
      const int cell = wi.cell_begin + tcl;
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        int nb = sd.nbr[(size_t)cell * 2 * DIM + 2 * te + s];
        if (nb >= sd.n_cells) {
          atomicOr(La.err, ERR_BAD_NEIGHBOR);
          nb = cell;
        }
        nbs[s] = nb;
      }
    }
  };
  // The item's neighbour arrays outside the block, issued by the first
  // thread of every (cell, direction) of the block (spread over the warps):
  // it copies the arrays of the two faces its direction's lines meet, whose
  // neighbour ids lookup_nb has just loaded.  bars[3] expects one arrival
  // from each of these CB * DIM threads per item (cells beyond a partial
  // item arrive without copies); each announces its bytes before its copies.
  const bool nb_issuer = tt == 0;
  auto issue_nb = [&](const WorkItem& wi, const int* nbs) {
    if (!nb_issuer) return;
    constexpr size_t fbytes = (size_t)N * sizeof(InT);
    // the 16-byte window around field f of cell nb: start and length
    auto window = [&](int nb, int f, size_t& w0) -> uint32_t {
      const size_t s0 = ((size_t)nb * F + f) * fbytes;
      w0 = s0 & ~(size_t)15;
      return (uint32_t)(((s0 + fbytes + 15) & ~(size_t)15) - w0);
    };
    const SolveDesc* sdp = La.solves ? La.solves + wi.solve : &La.single;
    const unsigned char* Xg = static_cast<const unsigned char*>(sdp->X);
    size_t wu[2] = {0, 0}, wp[2] = {0, 0};
    uint32_t lu[2] = {0, 0}, lp[2] = {0, 0};
    uint32_t bytes = 0;
    if (tcl < wi.n_cells) {
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int nb = nbs[s];
        const int nl = nb - wi.cell_begin;
        if (nb >= 0 && !(nl >= 0 && nl < wi.n_cells)) {
          lu[s] = window(nb, te, wu[s]);
          lp[s] = window(nb, DIM, wp[s]);
          bytes += lu[s] + lp[s];
        }
      }
    }
    if (bytes > 0) mbar_add_tx(&bars[3], bytes);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (lu[s] > 0) {
        const int q = tcl * 2 * DIM + 2 * te + s;
        bulk_g2s(sNb + (size_t)(2 * q) * NB_SLOT, Xg + wu[s], lu[s], &bars[3]);
        bulk_g2s(sNb + (size_t)(2 * q + 1) * NB_SLOT, Xg + wp[s], lp[s], &bars[3]);
      }
    }
    mbar_arrive(&bars[3]);
  };
  // Neighbour lines (u_e and p, both sides) of item wi that are not in the
  // item's own block: asynchronous copies from L2 into this thread's slot.
  auto prefetch_nb = [&](const WorkItem& wi, const SolveDesc& sd, int* nbs) {
    lookup_nb(wi, sd, nbs);
    const InT* Xg = static_cast<const InT*>(sd.X);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int nb = nbs[s];
      const int nl = nb - wi.cell_begin;
      if (tcl < wi.n_cells && nb >= 0 && !(nl >= 0 && nl < wi.n_cells)) {
        const size_t o = (size_t)nb * F * N;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const size_t iu = o + te * N + tbase + j * tstr, ip = o + DIM * N + tbase + j * tstr;
          cp_async<sizeof(InT)>(nslot + ((2 * s) * NP + j) * nstride, Xg + iu);
          cp_async<sizeof(InT)>(nslot + ((2 * s + 1) * NP + j) * nstride, Xg + ip);
        }
      }
    }
    cp_async_commit();
  };

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    mbar_init(&bars[3], CB * DIM);
    fence_barrier_init();
  }
  __syncthreads();
  if (ca.tma && threadIdx.x == 0 && (int)blockIdx.x < La.n_work) issue(La.work[blockIdx.x], 0);
  int nbs[2];

  uint32_t phase = 0;  // bit b: parity of the next wait on buffer b
  int it = 0;
  bool prev_a_ok = true;  // the previous item's accumulator copy arrived
  bool prev_nb_ok = true;  // this thread saw the previous item's neighbour arrays arrive
  int nb_last = -1;        // item index of the last neighbour phase issued
  bool nb_fail = false;    // a neighbour wait of the previous item gave up
  for (int w = blockIdx.x; w < La.n_work; w += gridDim.x, ++it) {
    const int b = it & 1;
    const bool has_next = w + (int)gridDim.x < La.n_work;
    const WorkItem wi = La.work[w];
    // by value: the fields live in registers instead of being re-read after
    // every store (a reference could alias the output arrays)
    const SolveDesc sd = La.solves ? La.solves[wi.solve] : La.single;
    const int nc = wi.n_cells;
    InT* sX = reinterpret_cast<InT*>(smem_cart + lay.X + b * xstride);
    double* sA = reinterpret_cast<double*>(smem_cart + lay.A + (a_single ? 0 : b * astride));
    // accumulator value of a staged point: FP64 / float pair, or the pair
    // assembled from the hi (X) and lo arrays
    auto aval = [&](int idx) -> double {
      if constexpr (!stage_a) {
        return 0.0;
      } else if constexpr (LO_IN) {
        return ff_pack(static_cast<float>(sX[idx]), reinterpret_cast<const float*>(sA)[idx]);
      } else {
        return sA[idx];
      }
    };
    // one value's outputs: next stage input and accumulator / new state
    auto store_out = [&](size_t g, OutT xn, double an) {
      if constexpr (EpiTraits<EPI>::writes_x) static_cast<OutT*>(sd.Xout)[g] = xn;
      if constexpr (LO_OUT) {
        reinterpret_cast<float*>(sd.Aout)[g] = ff_lo(an);
      } else {
        sd.Aout[g] = an;
      }
    };
    bool a_ok = true, a_ready = !(ca.tma && a_single);
    auto wait_a = [&]() {
      if (!a_ready) {
        a_ok = mbar_wait(&bars[2], (uint32_t)it & 1u);
        a_ready = true;
      }
    };
    // per-cell constants (prepared on the host, see ew_create)
    {
      const Real* gc = static_cast<const Real*>(sd.cellc) + (size_t)wi.cell_begin * kCellConsts;
      for (int i = threadIdx.x; i < nc * kCellConsts; i += blockDim.x) sCell[i] = load_nc(gc + i);
    }
    const bool tactive = tcl < nc;
    // this item's non-local neighbour lines: in flight during the bulk-copy
    // wait and the own-line contractions, awaited just before the fluxes
    // (issuing them one phase earlier, during the previous item's pressure
    // phase, measured 3-4% slower)
    if (nb_bulk) {
      lookup_nb(wi, sd, nbs);
      // a new phase only once every wait of the previous one ended in time
      // (known to every thread from the previous item's last barrier)
      if (!nb_fail) {
        issue_nb(wi, nbs);
        nb_last = it;
      }
    } else {
      prefetch_nb(wi, sd, nbs);
    }
    if (ca.tma) {
      const bool ok = mbar_wait(&bars[b], (phase >> b) & 1u);
      phase ^= (1u << b);
      // One barrier both ends the previous item (its pressure phase read the
      // accumulator buffer and, for float-pair input, the other X buffer)
      // and starts this one (cell constants written, X landed).
      if (__syncthreads_or(!ok || !prev_a_ok || !prev_nb_ok)) {
        // give up on this CTA's remaining items: wait (bounded) for the
        // copies still in flight, then leave
        if (threadIdx.x == 0) {
          atomicOr(La.err, ERR_WAIT_TIMEOUT);
          if (!ok) mbar_wait(&bars[b], ((phase >> b) & 1u) ^ 1u);
          if (a_single && it > 0) mbar_wait(&bars[2], (uint32_t)(it - 1) & 1u);
          // neighbour arrays: the last phase issued (phases end in order)
          if (nb_bulk && nb_last >= 0) mbar_wait(&bars[3], (uint32_t)nb_last & 1u);
        }
        cp_async_wait_all();
        prev_a_ok = true;
        prev_nb_ok = true;
        break;
      }
      if (threadIdx.x == 0) {
        fence_proxy_async();
        // the next item into the other buffer, and this item's accumulator
        // (single buffer, needed only by the epilogue)
        if (has_next) issue(La.work[w + gridDim.x], b ^ 1);
        if (a_single) issue_a(wi);
      }
    } else {
      __syncthreads();  // the previous item is done with the buffers
      const size_t c0 = (size_t)wi.cell_begin * F * N;
      if (stage_x) {
        const InT* gx = static_cast<const InT*>(sd.X) + c0;
        for (int i = threadIdx.x; i < nc * F * N; i += blockDim.x) sX[i] = gx[i];
      }
      if constexpr (stage_a && LO_IN) {
        const float* ga = reinterpret_cast<const float*>(sd.A) + c0;
        for (int i = threadIdx.x; i < nc * F * N; i += blockDim.x) reinterpret_cast<float*>(sA)[i] = ga[i];
      } else if constexpr (stage_a) {
        const double* ga = sd.A + c0;
        for (int i = threadIdx.x; i < nc * F * N; i += blockDim.x) sA[i] = ga[i];
      }
      __syncthreads();
    }
    if constexpr (CONV) {
      // FP32 operator on FP64 values: each staged value is converted once,
      // in place, to a float pair (hi in the low word is the operator input).
      // MIX_S1 splits the accumulator exactly, hi + lo, and continues from
      // the pair like the middle stages.
      const int tot = nc * F * N;
      if constexpr (EPI == EPI_MIX_S1) {
        for (int i = threadIdx.x; i < tot; i += blockDim.x) {
          float hi, lo;
          f64_split(sA[i], hi, lo);
          sA[i] = ff_pack(hi, lo);
        }
      }
      if (stage_x) {
        double* sX64 = reinterpret_cast<double*>(sX);
        if constexpr (is_ff_v<Real>) {
          // compensated operator: the exact pair of each value
          for (int i = threadIdx.x; i < tot; i += blockDim.x) {
            float hi, lo;
            f64_split(sX64[i], hi, lo);
            sX64[i] = ff_pack(hi, lo);
          }
        } else {
          for (int i = threadIdx.x; i < tot; i += blockDim.x) sX64[i] = ff_pack(f64_to_f32(sX64[i]), 0.f);
        }
      }
      // these generic writes precede the bulk copy that refills the buffer
      fence_proxy_async();
      __syncthreads();
    }

    // ---------------------------------------------------------- line phase
    // stage input values as Real, from the X buffer or (X == A) the A buffer
    auto xval = [&](int idx) -> Real {
      if constexpr (is_ff_v<InT>) {
        // float pairs: staged on their own, or (X == A, the first stage of a
        // step from a float-pair state) in the accumulator's buffer
        return stage_x ? sX[idx] : reinterpret_cast<const FF*>(sA)[idx];
      } else if constexpr (sizeof(InT) == 4) {
        return sX[idx];
      } else if constexpr (CONV && is_ff_v<Real>) {
        const float* p = reinterpret_cast<const float*>(stage_x ? static_cast<const void*>(sX)
                                                                : static_cast<const void*>(sA));
        return Real(p[2 * idx], p[2 * idx + 1]);
      } else if constexpr (CONV) {
        return reinterpret_cast<const float*>(stage_x ? static_cast<const void*>(sX)
                                                      : static_cast<const void*>(sA))[2 * idx];
      } else {
        const double* src = stage_x ? reinterpret_cast<const double*>(sX) : sA;
        return to_real<Real>(src[idx]);
      }
    };
    const Real bf = static_cast<Real>(sd.bf);
    {
      const int cl = tcl, e = te, base = tbase, str = tstr;
      if (tactive) {
        const Real* cst = sCell + cl * kCellConsts;
        const int xo = cl * F * N;
        Real ku[NP], kp[NP];
        if constexpr (is_ff_v<Real>) {
          // Compensated arithmetic with anchored sums (ew_ff.cuh): every
          // line sum -- traces, derivative contractions with the face lifts
          // folded in -- is accumulated on an anchor derived from the
          // largest |value| on its line; the flux algebra uses unnormalised
          // pairs.  The fluxes are written through q = t_p - lambda:
          //   lift of u_e: -nrm q,  lift of p: -n.u - tau q,
          // so that k_u = (-bf/h rho^-1) (D p + W G_u) and
          // k_p = (bf/h rho c^2) (D^T u + W G_p).
          const FfBounds& FB = c_ff_bounds;
          const Real rho_inv = cst[0], rc2 = cst[1], tau_p = cst[2], itau = cst[3], ih = cst[4 + e];
          FF xu[NP], xp[NP];
#pragma unroll
          for (int j = 0; j < NP; ++j) {
            xu[j] = xval(xo + e * N + base + j * str);
            xp[j] = xval(xo + DIM * N + base + j * str);
          }
          FF eu[HA], ou[HA], ep[HA], op[HA];
#pragma unroll
          for (int j = 0; j < H; ++j) {
            eu[j] = ffu_add(xu[j], xu[NP - 1 - j]);
            ou[j] = ffu_sub(xu[j], xu[NP - 1 - j]);
            ep[j] = ffu_add(xp[j], xp[NP - 1 - j]);
            op[j] = ffu_sub(xp[j], xp[NP - 1 - j]);
          }
          const FF um = (NP % 2) ? xu[NP / 2] : FF(0.f), pm = (NP % 2) ? xp[NP / 2] : FF(0.f);
          // own traces at x_e = 0 (s + a) and x_e = 1 (s - a)
          FF tu[2], tp[2];
          {
            float bsu = 0.f, bau = 0.f, bsp = 0.f, bap = 0.f;
            if constexpr (NP % 2 == 1) {
              bsu = FB.aLmid * fabsf(um.hi);
              bsp = FB.aLmid * fabsf(pm.hi);
            }
#pragma unroll
            for (int j = 0; j < H; ++j) {
              bsu = __fmaf_rn(FB.aLs[j], fabsf(eu[j].hi), bsu);
              bau = __fmaf_rn(FB.aLa[j], fabsf(ou[j].hi), bau);
              bsp = __fmaf_rn(FB.aLs[j], fabsf(ep[j].hi), bsp);
              bap = __fmaf_rn(FB.aLa[j], fabsf(op[j].hi), bap);
            }
            const float Su = anchor_for(fmaxf(bsu, bau)), Sp = anchor_for(fmaxf(bsp, bap));
            AAcc su = aa_init(Su), au = aa_init(Su), sp = aa_init(Sp), ap = aa_init(Sp);
            if constexpr (NP % 2 == 1) {
              aa_add(su, B.Lmid, um);
              aa_add(sp, B.Lmid, pm);
            }
#pragma unroll
            for (int j = 0; j < H; ++j) {
              aa_add(su, B.Ls[j], eu[j]);
              aa_add(au, B.La[j], ou[j]);
              aa_add(sp, B.Ls[j], ep[j]);
              aa_add(ap, B.La[j], op[j]);
            }
            aa_pm(au, su, Su, tu[0], tu[1]);
            aa_pm(ap, sp, Sp, tp[0], tp[1]);
          }
          if (nb_bulk) {
            if (!mbar_wait(&bars[3], (uint32_t)it & 1u)) {
              atomicOr(La.err, ERR_WAIT_TIMEOUT);
              prev_nb_ok = false;
            }
          } else {
            cp_async_wait_all();
          }
          // lift inputs of both faces
          FF Gu[2], Gp[2];
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            const FF un_p = s ? tu[1] : FF(-tu[0].hi, -tu[0].lo);  // nrm . u on this side
            const int nb = nbs[s];
            FF q;  // t_p - lambda
            if (nb >= 0) {
              const int nl = nb - wi.cell_begin;
              FF nu[NP], np_[NP];
              if (!(nl >= 0 && nl < nc) && nb_bulk) {
                const unsigned char* slot = sNb + (size_t)(2 * (cl * 2 * DIM + 2 * e + s)) * NB_SLOT;
                const InT* pu = reinterpret_cast<const InT*>(slot + nb_rem(nb, e)) + base;
                const InT* pp = reinterpret_cast<const InT*>(slot + NB_SLOT + nb_rem(nb, DIM)) + base;
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                  nu[j] = to_real<FF>(pu[j * str]);
                  np_[j] = to_real<FF>(pp[j * str]);
                }
              } else if (!(nl >= 0 && nl < nc)) {
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                  nu[j] = to_real<FF>(nslot[((2 * s) * NP + j) * nstride]);
                  np_[j] = to_real<FF>(nslot[((2 * s + 1) * NP + j) * nstride]);
                }
              } else {
                const int no = nl * F * N;
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                  nu[j] = xval(no + e * N + base + j * str);
                  np_[j] = xval(no + DIM * N + base + j * str);
                }
              }
              float bnu = 0.f, bnp = 0.f;
#pragma unroll
              for (int j = 0; j < NP; ++j) {
                bnu = __fmaf_rn(FB.aL[1 - s][j], fabsf(nu[j].hi), bnu);
                bnp = __fmaf_rn(FB.aL[1 - s][j], fabsf(np_[j].hi), bnp);
              }
              const float Snu = anchor_for(bnu), Snp = anchor_for(bnp);
              AAcc vu = aa_init(Snu), vp = aa_init(Snp);
#pragma unroll
              for (int j = 0; j < NP; ++j) {
                aa_add(vu, B.L[1 - s][j], nu[j]);
                aa_add(vp, B.L[1 - s][j], np_[j]);
              }
              const FF vU = aa_value(vu, Snu), vP = aa_value(vp, Snp);
              const Real tau_m = cst[7 + 2 * (2 * e + s)];
              const Real tau_inv = cst[8 + 2 * (2 * e + s)];
              // un_m = -nrm vu; t_p - lambda = (tau_m (t_p - v_p) - (un_p + un_m)) / (tau_p + tau_m)
              const FF un_m = s ? FF(-vU.hi, -vU.lo) : vU;
              q = ffu_mul(ffu_sub(ffu_mul(tau_m, ffu_sub(tp[s], vP)), ffu_add(un_p, un_m)), tau_inv);
            } else {
              const int id = -nb;
              if (id == EW_BC_SOFT_WALL_ID) {
                // lambda = un_p / tau + t_p
                const FF t = ffu_mul(un_p, itau);
                q = FF(-t.hi, -t.lo);
              } else if (id == EW_BC_ABSORBING_ID) {
                // lambda = (t_p + un_p / tau) / 2
                const FF t = ffu_sub(tp[s], ffu_mul(un_p, itau));
                q = FF(0.5f * t.hi, 0.5f * t.lo);
              } else {
                if (id != EW_BC_HARD_WALL_ID) atomicOr(La.err, ERR_BAD_BOUNDARY_ID);
                q = tp[s];  // lambda = 0
              }
            }
            Gu[s] = s ? FF(-q.hi, -q.lo) : q;
            const FF g = ffu_add(un_p, ffu_mul(tau_p, q));
            Gp[s] = FF(-g.hi, -g.lo);
          }
          const FF Gsu = ffu_add(Gu[0], Gu[1]), Gdu = ffu_sub(Gu[0], Gu[1]);
          const FF Gsp = ffu_add(Gp[0], Gp[1]), Gdp = ffu_sub(Gp[0], Gp[1]);
          const FF fh = ffu_norm(ffu_mul(ih, bf));
          const FF c1n = ffu_norm(ffu_mul(fh, rho_inv));
          const FF c1 = FF(-c1n.hi, -c1n.lo);
          const FF c2 = ffu_norm(ffu_mul(fh, rc2));
          // u_e: D p with the lifts of G_u; p: D^T u_e with the lifts of G_p
          // Each output pair (a_i, b_i) gets its own anchor from the row's
          // sum of |coefficient| |value| (float parts), which keeps the
          // anchor within a factor 4 of the row's largest partial sum.
          auto contract = [&](const EoMat<FF>& M, const float (*aP)[kEoMax], const float (*aQ)[kEoMax],
                              const float* amc, const float* amr, const FF* ev, const FF* ov, FF xm,
                              FF Gs, FF Gd, FF c, FF* k) {
            float ae[HA], ao[HA];
#pragma unroll
            for (int j = 0; j < H; ++j) {
              ae[j] = fabsf(ev[j].hi);
              ao[j] = fabsf(ov[j].hi);
            }
            const float ags = fabsf(Gs.hi), agd = fabsf(Gd.hi), axm = fabsf(xm.hi);
#pragma unroll
            for (int i = 0; i < H; ++i) {
              float ba = FB.aWa[i] * agd, bb = FB.aWs[i] * ags;
              if constexpr (NP % 2 == 1) ba = __fmaf_rn(amc[i], axm, ba);
#pragma unroll
              for (int j = 0; j < H; ++j) {
                ba = __fmaf_rn(aP[i][j], ae[j], ba);
                bb = __fmaf_rn(aQ[i][j], ao[j], bb);
              }
              const float S = anchor_for(fmaxf(ba, bb));
              AAcc a = aa_init(S), b = aa_init(S);
#pragma unroll
              for (int j = 0; j < H; ++j) {
                aa_add(a, M.P[i][j], ev[j]);
                aa_add(b, M.Q[i][j], ov[j]);
              }
              if constexpr (NP % 2 == 1) aa_add(a, M.mid_col[i], xm);
              aa_add(a, B.Wa[i], Gd);
              aa_add(b, B.Ws[i], Gs);
              FF yp, ym;
              aa_pm(a, b, S, yp, ym);
              k[i] = ffu_mul(c, yp);
              k[NP - 1 - i] = ffu_mul(c, ym);
            }
            if constexpr (NP % 2 == 1) {
              float bm = FB.aWmid * ags;
#pragma unroll
              for (int j = 0; j < H; ++j) bm = __fmaf_rn(amr[j], ao[j], bm);
              const float S = anchor_for(bm);
              AAcc m = aa_init(S);
#pragma unroll
              for (int j = 0; j < H; ++j) aa_add(m, M.mid_row[j], ov[j]);
              aa_add(m, B.Wmid, Gs);
              k[H] = ffu_mul(c, aa_value(m, S));
            }
          };
          contract(B.D, FB.aDP, FB.aDQ, FB.aDmc, FB.aDmr, ep, op, pm, Gsu, Gdu, c1, ku);
          contract(B.Dt, FB.aTP, FB.aTQ, FB.aTmc, FB.aTmr, eu, ou, um, Gsp, Gdp, c2, kp);
        } else {
          const Real rho_inv = cst[0], rc2 = cst[1], tau_p = cst[2], itau = cst[3], ih = cst[4 + e];
          Real xu[NP], xp[NP];
#pragma unroll
          for (int j = 0; j < NP; ++j) {
            xu[j] = xval(xo + e * N + base + j * str);
            xp[j] = xval(xo + DIM * N + base + j * str);
          }
          Real eu[HA], ou[HA], ep[HA], op[HA];
#pragma unroll
          for (int j = 0; j < H; ++j) {
            eu[j] = xu[j] + xu[NP - 1 - j];
            ou[j] = xu[j] - xu[NP - 1 - j];
            ep[j] = xp[j] + xp[NP - 1 - j];
            op[j] = xp[j] - xp[NP - 1 - j];
          }
          const Real um = (NP % 2) ? xu[NP / 2] : Real(0);
          const Real pm = (NP % 2) ? xp[NP / 2] : Real(0);
          // own traces at x_e = 0 (side 0) and x_e = 1 (side 1)
          Real su = (NP % 2) ? B.Lmid * um : Real(0), au = Real(0);
          Real sp = (NP % 2) ? B.Lmid * pm : Real(0), ap = Real(0);
#pragma unroll
          for (int j = 0; j < H; ++j) {
            su = mac(su, B.Ls[j], eu[j]);
            au = mac(au, B.La[j], ou[j]);
            sp = mac(sp, B.Ls[j], ep[j]);
            ap = mac(ap, B.La[j], op[j]);
          }
          su = end_sum(su);
          au = end_sum(au);
          sp = end_sum(sp);
          ap = end_sum(ap);
          const Real tu[2] = {su + au, su - au};
          const Real tp[2] = {sp + ap, sp - ap};
          if (nb_bulk) {
            // the item's neighbour arrays (bulk copies on bars[3])
            if (!mbar_wait(&bars[3], (uint32_t)it & 1u)) {
              atomicOr(La.err, ERR_WAIT_TIMEOUT);
              prev_nb_ok = false;
            }
          } else {
            cp_async_wait_all();  // this thread's neighbour lines
          }
          // fluxes at both ends (without the face JxW)
          Real Fu[2], Fp[2];
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            const Real nrm = s ? Real(1) : Real(-1);
            const Real un_p = nrm * tu[s];
            const int nb = nbs[s];
            Real lambda;
            if (nb >= 0) {
              const int nl = nb - wi.cell_begin;
              Real vu = Real(0), vp = Real(0);
              if (!(nl >= 0 && nl < nc) && nb_bulk) {
                // neighbour's line from its field arrays copied for this face
                const unsigned char* slot = sNb + (size_t)(2 * (cl * 2 * DIM + 2 * e + s)) * NB_SLOT;
                const InT* nu = reinterpret_cast<const InT*>(slot + nb_rem(nb, e)) + base;
                const InT* np_ = reinterpret_cast<const InT*>(slot + NB_SLOT + nb_rem(nb, DIM)) + base;
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                  const Real l = B.L[1 - s][j];
                  vu = mac(vu, l, to_real<Real>(nu[j * str]));
                  vp = mac(vp, l, to_real<Real>(np_[j * str]));
                }
              } else if (!(nl >= 0 && nl < nc)) {
                // neighbour's line from this thread's prefetch slot
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                  const Real l = B.L[1 - s][j];
                  vu = mac(vu, l, to_real<Real>(nslot[((2 * s) * NP + j) * nstride]));
                  vp = mac(vp, l, to_real<Real>(nslot[((2 * s + 1) * NP + j) * nstride]));
                }
              } else {
                // neighbour in this block: its trace on the opposite face, l_j(1-s)
                const int no = nl * F * N;
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                  const Real l = B.L[1 - s][j];
                  vu = mac(vu, l, xval(no + e * N + base + j * str));
                  vp = mac(vp, l, xval(no + DIM * N + base + j * str));
                }
              }
              vu = end_sum(vu);
              vp = end_sum(vp);
              const Real tau_m = cst[7 + 2 * (2 * e + s)];
              const Real tau_inv = cst[8 + 2 * (2 * e + s)];
              const Real un_m = -nrm * vu;
              lambda = (un_p + un_m + tau_p * tp[s] + tau_m * vp) * tau_inv;
            } else {
              const int id = -nb;
              if (id == EW_BC_SOFT_WALL_ID) {
                lambda = un_p * itau + tp[s];
              } else if (id == EW_BC_ABSORBING_ID) {
                lambda = Real(0.5) * tp[s] + Real(0.5) * un_p * itau;
              } else {
                if (id != EW_BC_HARD_WALL_ID) atomicOr(La.err, ERR_BAD_BOUNDARY_ID);
                lambda = Real(0);
              }
            }
            Fu[s] = (tp[s] - lambda) * rho_inv * nrm;
            Fp[s] = rc2 * (-un_p + tau_p * (lambda - tp[s]));
          }
          // derivative of p and weighted transpose derivative of u_e
          Real a1[HA + 1], b1[HA], a2[HA + 1], b2[HA];
          eo_apply<NP, Real>(B.D, ep, op, pm, a1, b1);
          eo_apply<NP, Real>(B.Dt, eu, ou, um, a2, b2);
          const Real Fsu = Fu[0] + Fu[1], Fdu = Fu[0] - Fu[1];
          const Real Fsp = Fp[0] + Fp[1], Fdp = Fp[0] - Fp[1];
          const Real fu = bf * ih, fpp = bf * ih;
#pragma unroll
          for (int i = 0; i < H; ++i) {
            // u_e: -rho^{-1} (D p)_i + lift; p: rho c^2 (Dt u)_i + lift
            const Real ua = -rho_inv * a1[i] + B.Wa[i] * Fdu;
            const Real ub = -rho_inv * b1[i] + B.Ws[i] * Fsu;
            ku[i] = fu * (ua + ub);
            ku[NP - 1 - i] = fu * (ub - ua);
            const Real pa = rc2 * a2[i] + B.Wa[i] * Fdp;
            const Real pb = rc2 * b2[i] + B.Ws[i] * Fsp;
            kp[i] = fpp * (pa + pb);
            kp[NP - 1 - i] = fpp * (pb - pa);
          }
          if constexpr (NP % 2 == 1) {
            ku[H] = fu * (-rho_inv * a1[H] + B.Wmid * Fsu);
            kp[H] = fpp * (rc2 * a2[H] + B.Wmid * Fsp);
          }
        }
        // pressure part of this direction to shared memory
#pragma unroll
        for (int i = 0; i < NP; ++i) sKp[(e * CB + cl) * N + base + i * str] = kp[i];
        // finish u_e on this line (x-lines are contiguous: paired stores)
        const size_t g0 = ((size_t)wi.cell_begin + cl) * F * N + e * N + base;
        const int l0 = xo + e * N + base;
        wait_a();
        if (a_ok) {
          const bool paired = NP % 2 == 0 && e == 0 &&
                              (reinterpret_cast<uintptr_t>(sd.Aout) & 15) == 0 &&
                              (reinterpret_cast<uintptr_t>(sd.Xout) & (2 * sizeof(OutT) - 1)) == 0;
#pragma unroll
          for (int i = 0; i < NP; i += 2) {
            OutT x0, x1 = OutT(0);
            double a0, a1 = 0.0;
            epi_value<EPI, Real, OutT>(sd, aval(l0 + i * str), ku[i], x0, a0);
            if (i + 1 < NP) epi_value<EPI, Real, OutT>(sd, aval(l0 + (i + 1) * str), ku[i + 1], x1, a1);
            if (paired) {
              if constexpr (EpiTraits<EPI>::writes_x) store2(static_cast<OutT*>(sd.Xout) + g0 + i, x0, x1);
              if constexpr (LO_OUT)
                store2(reinterpret_cast<float*>(sd.Aout) + g0 + i, ff_lo(a0), ff_lo(a1));
              else
                store2(sd.Aout + g0 + i, a0, a1);
            } else {
              store_out(g0 + i * str, x0, a0);
              if (i + 1 < NP) store_out(g0 + (i + 1) * str, x1, a1);
            }
          }
        }
      }
    }
    // every wait on this item's neighbour arrays has ended here
    nb_fail = __syncthreads_or(!prev_nb_ok) != 0;
    // ---------------------------------------------------------- pressure
    const int src_local = sd.src_cell - wi.cell_begin;
    Real src_val = Real(0);
    if (src_local >= 0 && src_local < nc) {
      const double sv = sd.src_amp * ricker(*sd.time + sd.c_stage * sd.dt, sd.src_f0, sd.src_t0);
      if constexpr (is_ff_v<Real>)
        src_val = FF::from_double(sv);
      else
        src_val = static_cast<Real>(sv);
    }
    wait_a();
    for (int idx = threadIdx.x; a_ok && idx < nc * N; idx += blockDim.x) {
      const int cl = idx / N;
      const int q = idx - cl * N;
      Real k = sKp[cl * N + q];
#pragma unroll
      for (int e = 1; e < DIM; ++e) k += sKp[(e * CB + cl) * N + q];
      if (cl == src_local) k += src_val * static_cast<const Real*>(sd.src_w)[q];
      const size_t g = ((size_t)wi.cell_begin + cl) * F * N + DIM * N + q;
      const int lidx = cl * F * N + DIM * N + q;
      OutT xn;
      double an;
      epi_value<EPI, Real, OutT>(sd, aval(lidx), k, xn, an);
      store_out(g, xn, an);
    }
    // no end-of-item barrier: the next item's first barrier ends this one
    prev_a_ok = a_ok;
  }
  // the last item's copies: none may be in flight when the block ends
  if (__syncthreads_or(!prev_a_ok || !prev_nb_ok)) {
    if (threadIdx.x == 0) {
      atomicOr(La.err, ERR_WAIT_TIMEOUT);
      if (a_single && it > 0) mbar_wait(&bars[2], (uint32_t)(it - 1) & 1u);
      if (nb_bulk && nb_last >= 0) mbar_wait(&bars[3], (uint32_t)nb_last & 1u);
    }
  }
}

}  // namespace ew
