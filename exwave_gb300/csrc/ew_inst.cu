// ew_inst.cu -- instantiates the kernels for one (dimension, points per
// direction) pair, selected by -DEW_DIM and -DEW_NP, and exports their
// launchers through a table (one object file per pair, compiled in parallel).
#include "ew_basis.h"
#include "ew_cart.cuh"
#include "ew_kernels.cuh"
#include "ew_launch.h"
#include "ew_stage_tma.cuh"

#ifndef EW_DIM
#error "EW_DIM must be defined"
#endif
#ifndef EW_NP
#error "EW_NP must be defined"
#endif

namespace ew {
namespace {

constexpr int DIM = EW_DIM;
constexpr int NP = EW_NP;
constexpr int N = ipow_c(NP, DIM);
// The line kernel and the CK kernel keep whole cells in shared memory; in
// 3-D beyond 9^3 points (degree 8 and above) they do not fit, and those
// degrees run the generic stage kernel only (several points per thread).
constexpr bool LINE_OK = DIM == 2 || NP <= 8;
constexpr bool CK_OK = DIM == 2 || NP <= 8;
// threads of the generic stage kernel: one per point, or a cell of more
// than 512 points spread over PPT points per thread (one cell per block)
constexpr int STAGE_PPT = (N + 511) / 512;
constexpr int STAGE_THREADS_1 = ((N + STAGE_PPT - 1) / STAGE_PPT + 31) / 32 * 32;
inline int stage_threads(int cb) { return STAGE_PPT > 1 ? STAGE_THREADS_1 : cb * N; }

// Prefer the largest shared-memory carve-out: the kernels are limited by
// resident CTAs, not by L1 hits.
template <typename Kern>
void carveout(Kern kern) {
  cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                       (int)cudaSharedmemCarveoutMaxShared);
}

template <typename Kern>
cudaError_t run(Kern kern, const LaunchArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  carveout(kern);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<grid, block, smem, st>>>(a);
  return cudaGetLastError();
}

template <typename Kern>
int blocks_per_sm(Kern kern, int block, size_t smem) {
  carveout(kern);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, block, smem) != cudaSuccess) return 0;
  return nb;
}

template <typename Real, typename InT, typename OutT, bool CART>
struct StageK {
  static size_t smem(int cb) { return (size_t)OpSmem<DIM, NP, CART>(cb).end * sizeof(Real); }
  static size_t smem_staged(int cb) { return StagedSmem<DIM, NP>(cb, (int)sizeof(Real)).end; }
  // The staged kernel (bulk copies) serves curved cells when the input is
  // already in the compute type and every per-cell block is a multiple of
  // 16 bytes; the pointers are checked at launch.
  static bool staged_ok(int cb) {
    constexpr size_t F = DIM + 1;
    return !CART && std::is_same<Real, InT>::value && N <= 512 && (F * N * sizeof(Real)) % 16 == 0 &&
           (F * N * 8) % 16 == 0 && ((size_t)(1 << DIM) * DIM * sizeof(Real)) % 16 == 0 &&
           2 * DIM <= N && smem_staged(cb) <= 220 * 1024;
  }
  static bool aligned(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
  static cudaError_t launch(const LaunchArgs& a, int grid, cudaStream_t st) {
    const int cb = a.cells_per_block;
    if constexpr (!CART && std::is_same<Real, InT>::value) {
      const SolveDesc& s = a.single;
      if (staged_ok(cb) && a.solves == nullptr && aligned(s.X) && aligned(s.geo) && aligned(s.mat) &&
          (s.mode == MODE_APPLY || aligned(s.A)))
        return run(stage_kernel_staged<DIM, NP, Real, OutT>, a, grid, cb * N, smem_staged(cb), st);
    }
    return run(stage_kernel<DIM, NP, Real, InT, OutT, CART>, a, grid, stage_threads(cb), smem(cb), st);
  }
  static int occupancy(int cb) {
    if constexpr (!CART && std::is_same<Real, InT>::value) {
      if (staged_ok(cb))
        return blocks_per_sm(stage_kernel_staged<DIM, NP, Real, OutT>, cb * N, smem_staged(cb));
    }
    return blocks_per_sm(stage_kernel<DIM, NP, Real, InT, OutT, CART>, stage_threads(cb), smem(cb));
  }
};

template <typename Real, typename InT, typename OutT, bool CART, bool POST, bool SPEC = true>
struct CkK {
  static size_t smem(int cb) {
    return (size_t)CkSmem<DIM, NP, CART>(cb, ck_in_words<Real, InT>()).end * sizeof(Real);
  }
  static cudaError_t launch(const LaunchArgs& a, int grid, cudaStream_t st) {
    const int cb = a.cells_per_block;
    return run(ck_kernel<DIM, NP, Real, InT, OutT, CART, POST, SPEC>, a, grid, cb * N, smem(cb), st);
  }
  static int occupancy(int cb) {
    return blocks_per_sm(ck_kernel<DIM, NP, Real, InT, OutT, CART, POST, SPEC>, cb * N, smem(cb));
  }
};

template <typename Real, typename InT, int EPI>
struct CartK {
  static constexpr bool SA = EpiTraits<EPI>::stage_a;
  // Block size: one thread per (cell, direction, line).  (Padding the
  // compensated kernel's 7-warp blocks to 8 warps, to spread two blocks'
  // warps evenly over the SM's schedulers, measured 5% slower at k = 5.)
  static int threads(int cb) { return cb * DIM * ipow_c(NP, DIM - 1); }
  static size_t smem(int cb, int sx) {
    return CartSmem<DIM, NP, Real, InT, EpiTraits<EPI>::a_elem>(cb, sx != 0, SA).end;
  }
  static cudaError_t launch(const LaunchArgs& a, int sx, int tma, int nb_lines, int grid,
                            cudaStream_t st) {
    CartArgs ca;
    ca.la = a;
    ca.stage_x = sx;
    ca.tma = tma;
    ca.nb_lines = nb_lines;
    const int cb = a.cells_per_block;
    const size_t sm = smem(cb, sx);
    auto kern = stage_cart_kernel<DIM, NP, Real, InT, EPI>;
    carveout(kern);
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return e;
    }
    kern<<<grid, threads(cb), sm, st>>>(ca);
    return cudaGetLastError();
  }
  static int occupancy(int cb, int sx) {
    return blocks_per_sm(stage_cart_kernel<DIM, NP, Real, InT, EPI>, threads(cb), smem(cb, sx));
  }
};

template <class K>
void fill_cart(CartEntry& e) {
  e.launch = &K::launch;
  e.occupancy = &K::occupancy;
  e.smem = &K::smem;
}

cudaError_t set_constants(const double* w, const double* D, const double* L0, const double* L1) {
  const CartBasis<double> cd = make_cart_basis(NP, w, D, L0, L1);
  const CartBasis<float> cf = cast_basis<float>(cd);
  cudaError_t e = cudaMemcpyToSymbol(c_cart_d, &cd, sizeof(cd));
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(c_cart_f, &cf, sizeof(cf));
  if (e != cudaSuccess) return e;
  const CartBasis<FF> cff = cast_basis<FF>(cd);
  e = cudaMemcpyToSymbol(c_cart_ff, &cff, sizeof(cff));
  if (e != cudaSuccess) return e;
  const FfBounds fb = make_ff_bounds(cd);
  e = cudaMemcpyToSymbol(c_ff_bounds, &fb, sizeof(fb));
  if (e != cudaSuccess) return e;
  // the CK kernel's multilevel tables, in each compute type
  static_assert(basis_total(NP) <= kCkBasisMax, "CK table larger than its constant array");
  const std::vector<double> bt = basis_table(NP);
  if ((int)bt.size() != basis_total(NP)) return cudaErrorInvalidValue;
  std::vector<float> btf(bt.size());
  std::vector<FF> btff(bt.size());
  for (size_t i = 0; i < bt.size(); ++i) {
    btf[i] = static_cast<float>(bt[i]);
    btff[i] = FF::from_double(bt[i]);
  }
  e = cudaMemcpyToSymbol(c_ckb_d, bt.data(), bt.size() * sizeof(double));
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(c_ckb_f, btf.data(), btf.size() * sizeof(float));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_ckb_ff, btff.data(), btff.size() * sizeof(FF));
}

template <class K>
void fill(KernelEntry& e) {
  e.launch = &K::launch;
  e.occupancy = &K::occupancy;
  e.smem = &K::smem;
}

}  // namespace

#define EW_CAT2(a, b, c) a##b##_##c
#define EW_CAT(a, b, c) EW_CAT2(a, b, c)
#define EW_TABLE_FN EW_CAT(kernel_table_d, EW_DIM, EW_NP)

void EW_TABLE_FN(KernelTable& t) {
  t.dim = DIM;
  t.np = NP;
  t.points = N;
  t.lines = DIM * ipow_c(NP, DIM - 1);
  t.set_constants = &set_constants;
  if constexpr (LINE_OK) {
    fill_cart<CartK<double, double, EPI_APPLY>>(t.cart[CV_F64_APPLY]);
    fill_cart<CartK<double, double, EPI_F64_MID>>(t.cart[CV_F64_MID]);
    fill_cart<CartK<double, double, EPI_F64_LAST>>(t.cart[CV_F64_LAST]);
    fill_cart<CartK<float, double, EPI_APPLY>>(t.cart[CV_MIX_APPLY64]);
    fill_cart<CartK<float, double, EPI_MIX_S1>>(t.cart[CV_MIX_S1]);
    fill_cart<CartK<float, float, EPI_APPLY>>(t.cart[CV_MIX_APPLY32]);
    fill_cart<CartK<float, float, EPI_MIX_MID>>(t.cart[CV_MIX_MID]);
    fill_cart<CartK<float, float, EPI_MIX_LAST>>(t.cart[CV_MIX_LAST]);
    fill_cart<CartK<float, float, EPI_MIX_UPD>>(t.cart[CV_MIX_UPD]);
    fill_cart<CartK<float, float, EPI_MIX_S1_FF>>(t.cart[CV_MIX_S1_FF]);
    fill_cart<CartK<float, float, EPI_MIX_LAST_FF>>(t.cart[CV_MIX_LAST_FF]);
    fill_cart<CartK<FF, double, EPI_APPLY>>(t.cart[CV_FF_APPLY64]);
    fill_cart<CartK<FF, double, EPI_MIX_S1>>(t.cart[CV_FF_S1]);
    fill_cart<CartK<FF, FF, EPI_MIX_MID>>(t.cart[CV_FF_MID]);
    fill_cart<CartK<FF, FF, EPI_MIX_LAST>>(t.cart[CV_FF_LAST]);
    fill_cart<CartK<FF, FF, EPI_MIX_UPD>>(t.cart[CV_FF_UPD]);
    fill_cart<CartK<FF, FF, EPI_APPLY>>(t.cart[CV_FF_APPLYFF]);
    fill_cart<CartK<FF, FF, EPI_FF_LAST_PAIR>>(t.cart[CV_FF_LAST_PAIR]);
  }
  // stage kernels: [variant][cart]; curved cells, and axis-aligned cells
  // where the line kernel is not built
  fill<StageK<double, double, double, false>>(t.stage[STAGE_F64][0]);
  fill<StageK<float, double, float, false>>(t.stage[STAGE_MIX_IN64][0]);
  fill<StageK<float, float, float, false>>(t.stage[STAGE_MIX_IN32][0]);
  fill<StageK<FF, double, FF, false>>(t.stage[STAGE_FF_IN64][0]);
  fill<StageK<FF, FF, FF, false>>(t.stage[STAGE_FF_INFF][0]);
  if constexpr (!LINE_OK) {
    fill<StageK<double, double, double, true>>(t.stage[STAGE_F64][1]);
    fill<StageK<float, double, float, true>>(t.stage[STAGE_MIX_IN64][1]);
    fill<StageK<float, float, float, true>>(t.stage[STAGE_MIX_IN32][1]);
    fill<StageK<FF, double, FF, true>>(t.stage[STAGE_FF_IN64][1]);
    fill<StageK<FF, FF, FF, true>>(t.stage[STAGE_FF_INFF][1]);
  }
  // CK kernels: [precision][cart][post]
  if constexpr (CK_OK) {
    fill<CkK<double, double, double, false, false>>(t.ck[0][0][0]);
    fill<CkK<double, double, double, false, true>>(t.ck[0][0][1]);
    fill<CkK<double, double, double, true, false>>(t.ck[0][1][0]);
    fill<CkK<double, double, double, true, true>>(t.ck[0][1][1]);
    fill<CkK<float, double, float, false, false>>(t.ck[1][0][0]);
    fill<CkK<float, double, float, false, true>>(t.ck[1][0][1]);
    fill<CkK<float, double, float, true, false>>(t.ck[1][1][0]);
    fill<CkK<float, double, float, true, true>>(t.ck[1][1][1]);
    fill<CkK<FF, double, FF, false, false>>(t.ck[2][0][0]);
    fill<CkK<FF, double, FF, false, true>>(t.ck[2][0][1]);
    fill<CkK<FF, double, FF, true, false>>(t.ck[2][1][0]);
    fill<CkK<FF, double, FF, true, true>>(t.ck[2][1][1]);
    // without spectral evaluation (no degree reduction; from k = 4 on the
    // two differ)
    if constexpr (NP >= 5) {
      fill<CkK<double, double, double, false, false, false>>(t.ck_full[0][0][0]);
      fill<CkK<double, double, double, false, true, false>>(t.ck_full[0][0][1]);
      fill<CkK<double, double, double, true, false, false>>(t.ck_full[0][1][0]);
      fill<CkK<double, double, double, true, true, false>>(t.ck_full[0][1][1]);
      fill<CkK<float, double, float, false, false, false>>(t.ck_full[1][0][0]);
      fill<CkK<float, double, float, false, true, false>>(t.ck_full[1][0][1]);
      fill<CkK<float, double, float, true, false, false>>(t.ck_full[1][1][0]);
      fill<CkK<float, double, float, true, true, false>>(t.ck_full[1][1][1]);
      fill<CkK<FF, double, FF, false, false, false>>(t.ck_full[2][0][0]);
      fill<CkK<FF, double, FF, false, true, false>>(t.ck_full[2][0][1]);
      fill<CkK<FF, double, FF, true, false, false>>(t.ck_full[2][1][0]);
      fill<CkK<FF, double, FF, true, true, false>>(t.ck_full[2][1][1]);
    }
  }
}

}  // namespace ew
