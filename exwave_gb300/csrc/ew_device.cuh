// ew_device.cuh -- device-side building blocks of the DG wave operator.
//
// Discretisation: the DG space Q_k (k = NP-1) on quads/hexes, represented by
// its values at the NP^DIM Gauss points of each cell (collocation basis of
// QGauss(k+1)).  This is the space and quadrature of the reference
// (FE_DGQ(k) with QGauss(k+1), wave_equation_operations.cc:214-216); in this
// basis the mass matrix is diag(JxW) and the face trace along a line is one
// NP-point contraction with l_j(0) or l_j(1).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ew {

__host__ __device__ constexpr int ipow_c(int b, int e) { return e == 0 ? 1 : b * ipow_c(b, e - 1); }
__host__ __device__ __forceinline__ int ipow_rt(int b, int e) {
  int r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

// boundary ids (input_parameters.h:52-57 of the reference)
constexpr int EW_BC_SOFT_WALL_ID = 1;  // u.n = 0
constexpr int EW_BC_HARD_WALL_ID = 2;  // p = 0
constexpr int EW_BC_ABSORBING_ID = 3;  // first-order absorbing

enum Mode : int {
  MODE_APPLY = 0,    // Aout = k                       (operator only)
  MODE_RK_MID = 1,   // Xout = A + f1 k ; Aout = A + (f1+f2) k
  MODE_RK_LAST = 2   // Aout = A + f1 k
};

enum DeviceError : int {
  ERR_BAD_NEIGHBOR = 1,
  ERR_BAD_BOUNDARY_ID = 2,
  ERR_BAD_LAUNCH = 4
};

// Per-solve arguments of one operator launch.  The single-solve API passes
// one by value; batched launches read a device table indexed by the work
// item's solve number.
struct SolveDesc {
  const void* X;       // operator input (InT)  [cell][field][point]
  const double* A;     // accumulator / base state (FP64)
  void* Xout;          // next stage input (OutT), MODE_RK_MID
  double* Aout;        // MODE_APPLY: result; RK modes: accumulator out (may alias A)
  const int32_t* nbr;  // [cell][2*DIM]
  const void* geo;     // Real: Cartesian [cell][DIM] extents; else [cell][2^DIM][DIM] monomial
                       // coefficients of the multilinear map (see geom_general)
  const void* mat;     // Real [cell][2] = (rho, c)
  int64_t n_cells;
  double f1, f2;
  float f1f;           // f1 rounded (stage input of the mixed path)
  float f1_hi, f1_lo;  // f1 = hi + lo (RK_LAST increment of the mixed path)
  float fb_hi, fb_lo;  // f1 + f2 = hi + lo (RK_MID accumulator increment)
  float bf;            // +1: M^-1 A(u); -1: second ADER step sign (boundary_fac)
  int32_t mode;
  int32_t pad;
  const void* cellc;   // Real [cell][kCellConsts] constants of the Cartesian kernel
  // point source in the pressure equation (batched solves): amplitude *
  // Ricker(t) * phi_q(x_s) / JxW_q added to the pressure update of src_cell,
  // at the stage time t = *time + c_stage * dt
  const double* time;
  const void* src_w;   // Real [points]
  double src_amp, src_f0, src_t0, c_stage, dt;
  int32_t src_cell;    // -1: none
  int32_t pad2;
};

// Ricker wavelet (1 - 2 pi^2 f0^2 s^2) exp(-pi^2 f0^2 s^2), s = t - t0.
__device__ __forceinline__ double ricker(double t, double f0, double t0) {
  const double a = 9.869604401089358 * f0 * f0 * (t - t0) * (t - t0);
  return (1.0 - 2.0 * a) * exp(-a);
}

struct WorkItem {
  int32_t solve;
  int32_t cell_begin;
  int32_t n_cells;
  int32_t pad;
};

struct LaunchArgs {
  SolveDesc single;          // used when solves == nullptr
  const SolveDesc* solves;   // batched: device table
  const WorkItem* work;      // device work list
  int32_t n_work;
  int32_t cells_per_block;
  const void* basis;         // Real basis table (see basis_offsets)
  int* err;                  // device error flags (OR-ed)
  double dt;                 // ADER: time step of the Taylor integral
  // ADER Taylor coefficients, prepared on the host: dt, dt^2/2 and for the
  // recursive derivative j = s + 2 the factor -1/2 prod_{i=2}^{s+2}(-1/(i+1)) dt^(s+3)
  float ck_dt, ck_half_dt2;
  float ck_fac[12];
  double ck_dt_d, ck_half_dt2_d;
  double ck_fac_d[12];
};

// ---------------------------------------------------------------- basis table
// Level r (ADER degree reduction) has m = NP - 2r points.  For each level:
// x[m], w[m], D[m*m] (D[i*m+j] = l_j'(x_i)), L0[m], L1[m]; for r >= 1 also
// P[m * m_prev] (L2 projection from level r-1) and E[m_prev * m]
// (interpolation back to level r-1).
__host__ __device__ constexpr int level_size(int m, int m_prev) {
  return 4 * m + m * m + (m_prev > 0 ? 2 * m * m_prev : 0);
}
__host__ __device__ constexpr int basis_offset(int NP, int r) {
  return r == 0 ? 0
                : basis_offset(NP, r - 1) + level_size(NP - 2 * (r - 1), r - 1 == 0 ? 0 : NP - 2 * (r - 2));
}
__host__ __device__ constexpr int n_levels(int NP) { return (NP + 1) / 2; }
__host__ __device__ constexpr int basis_total(int NP) { return basis_offset(NP, n_levels(NP)); }

template <typename Real>
struct Level {
  const Real* x;
  const Real* w;
  const Real* D;
  const Real* L0;
  const Real* L1;
  const Real* P;  // (m x m_prev), nullptr at r = 0
  const Real* E;  // (m_prev x m)
  int m;
};

template <typename Real>
__device__ __forceinline__ Level<Real> get_level(const Real* base, int NP, int r) {
  Level<Real> L;
  const int m = NP - 2 * r;
  const Real* p = base + basis_offset(NP, r);
  L.m = m;
  L.x = p;
  L.w = p + m;
  L.D = p + 2 * m;
  L.L0 = p + 2 * m + m * m;
  L.L1 = p + 3 * m + m * m;
  if (r > 0) {
    const int mp = m + 2;
    L.P = p + 4 * m + m * m;
    L.E = L.P + m * mp;
  } else {
    L.P = nullptr;
    L.E = nullptr;
  }
  return L;
}

// ---------------------------------------------------------------- conversions
// FP64 <-> FP32 conversions done on the integer pipe.  GB300 executes FP64
// arithmetic and FP64 conversions at a small fraction of its FP32 rate; the
// mixed-precision epilogue needs two conversions per DoF and stage, so they
// are done with integer operations on the bit patterns (round to nearest,
// ties away; results below FP32's normal range flush to zero).
__device__ __forceinline__ float f64_to_f32(double a) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const unsigned long long r = (b & 0x7fffffffffffffffull) + (1ull << 28);
  const int e = (int)(r >> 52) - 896;
  const unsigned int m = (unsigned int)(r >> 29) & 0x7fffffu;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((unsigned int)e << 23) | m);
}

// Branch-free: a data-dependent early return lets the compiler if-convert
// a following FP64 add into two adds and a select.
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int sign = u & 0x80000000u;
  const unsigned int mag = u & 0x7fffffffu;
  const bool normal = mag >= 0x00800000u;
  const unsigned int hi = sign | (normal ? ((mag >> 3) + (896u << 20)) : 0u);
  const unsigned int lo = normal ? (mag << 29) : 0u;
  return __hiloint2double((int)hi, (int)lo);
}

// a = hi + lo with hi = f64_to_f32(a) and lo the nearest float to the exact
// remainder a - hi, on the integer pipes: the remainder is the part of the
// 53-bit significand below hi's 24 bits (at most 2^28 units of a's ulp, one
// int-to-float conversion), rescaled through its exponent field.  lo is
// flushed to zero where it would be subnormal (|lo| < 2^-126).
__device__ __forceinline__ void f64_split(double a, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const unsigned long long mag = b & 0x7fffffffffffffffull;
  const unsigned long long r = mag + (1ull << 28);
  const int e = (int)(r >> 52) - 896;
  const unsigned int m = (unsigned int)(r >> 29) & 0x7fffffu;
  const bool finite = e > 0 && e < 255;
  hi = __uint_as_float(e <= 0 ? sign : (e >= 255 ? (sign | 0x7f800000u) : (sign | ((unsigned int)e << 23) | m)));
  const long long rem = (long long)(mag - (r & ~((1ull << 29) - 1)));
  const unsigned int fb = __float_as_uint(__int2float_rn((int)rem));
  const int ef = (int)((fb >> 23) & 0xffu) + (int)(mag >> 52) - 1075;
  lo = __uint_as_float((finite && rem != 0 && ef > 0) ? (((fb & 0x807fffffu) | ((unsigned int)ef << 23)) ^ sign)
                                                      : sign);
}

template <typename T>
__device__ __forceinline__ T load_nc(const T* p) {
  return __ldg(p);
}

// ---------------------------------------------------------------- geometry
// Multilinear cell map in monomial form: x(xi) = sum_S C_S prod_{d in S} xi_d
// over the subsets S of the DIM directions (bit masks), C_S[i] at
// C[S * DIM + i]; the host derives C from the 2^DIM vertices (deal.II
// lexicographic order) by C_S = sum_{T subset S} (-1)^{|S|-|T|} V_T.
// dx/dxi_j then needs one FMA per term: about 40 operations for J in 3-D
// instead of 120 from the vertices.  Returns det J and fills
// JiT[d][e] = d xi_e / d x_d.
template <int DIM, typename Real>
__device__ __forceinline__ Real geom_general(const Real* C, const Real* xi, Real JiT[DIM][DIM]) {
  constexpr int NV = 1 << DIM;
  Real J[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) J[i][j] = Real(0);
#pragma unroll
  for (int S = 1; S < NV; ++S) {
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      if (!((S >> j) & 1)) continue;
      Real prod = Real(1);
#pragma unroll
      for (int d = 0; d < DIM; ++d)
        if (d != j && ((S >> d) & 1)) prod *= xi[d];
#pragma unroll
      for (int i = 0; i < DIM; ++i) J[i][j] += C[S * DIM + i] * prod;
    }
  }
  if constexpr (DIM == 2) {
    const Real det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const Real id = Real(1) / det;
    JiT[0][0] = J[1][1] * id;
    JiT[0][1] = -J[1][0] * id;
    JiT[1][0] = -J[0][1] * id;
    JiT[1][1] = J[0][0] * id;
    return det;
  } else {
    const Real c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const Real c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const Real c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const Real c10 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    const Real c11 = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    const Real c12 = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    const Real c20 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    const Real c21 = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    const Real c22 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const Real det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    const Real id = Real(1) / det;
    JiT[0][0] = c00 * id; JiT[0][1] = c01 * id; JiT[0][2] = c02 * id;
    JiT[1][0] = c10 * id; JiT[1][1] = c11 * id; JiT[1][2] = c12 * id;
    JiT[2][0] = c20 * id; JiT[2][1] = c21 * id; JiT[2][2] = c22 * id;
    return det;
  }
}

// Geometry at a reference point of a cell whose geometry block (in shared
// memory) is either extents (Cartesian) or vertices.
template <int DIM, typename Real, bool CART>
__device__ __forceinline__ Real cell_geom(const Real* G, const Real* xi, Real JiT[DIM][DIM]) {
  if constexpr (CART) {
    Real det = Real(1);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
#pragma unroll
      for (int e = 0; e < DIM; ++e) JiT[d][e] = Real(0);
      JiT[d][d] = Real(1) / G[d];
      det *= G[d];
    }
    return det;
  } else {
    return geom_general<DIM, Real>(G, xi, JiT);
  }
}

template <int DIM, int NP>
__device__ __forceinline__ void split_point(int q, int* i) {
  i[0] = q % NP;
  if constexpr (DIM >= 2) i[1] = (q / NP) % NP;
  if constexpr (DIM >= 3) i[2] = q / (NP * NP);
}

// tangential face index of point i for a face in direction e
template <int DIM, int NP>
__device__ __forceinline__ int face_index(const int* i, int e) {
  if constexpr (DIM == 2) {
    return i[1 - e];
  } else {
    const int a = (e == 0) ? 1 : 0;
    const int b = (e == 2) ? 1 : 2;
    return i[a] + NP * i[b];
  }
}

// base point (i_e = 0) and tangential reference coordinates of face point t
template <int DIM, int NP>
__device__ __forceinline__ int face_base(int e, int t, int* ti) {
  if constexpr (DIM == 2) {
    const int d0 = 1 - e;
    ti[d0] = t;
    ti[e] = 0;
    return t * (d0 == 0 ? 1 : NP);
  } else {
    const int a = (e == 0) ? 1 : 0;
    const int b = (e == 2) ? 1 : 2;
    const int ta = t % NP, tb = t / NP;
    ti[a] = ta;
    ti[b] = tb;
    ti[e] = 0;
    const int sa = (a == 0) ? 1 : NP;       // a is 0 or 1
    const int sb = (b == 1) ? NP : NP * NP;  // b is 1 or 2
    return ta * sa + tb * sb;
  }
}

// shared-memory address of a generic pointer into shared memory
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Ampere-style asynchronous copies (LDGSTS) of 4 or 8 bytes into shared memory.
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src),
               "n"(BYTES)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

}  // namespace ew
