// ew_launch.h -- table of kernel launchers per (dimension, degree), filled
// by the instantiation units (ew_inst.cu compiled once per pair).
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

#include "ew_device.cuh"

namespace ew {

enum StageVariant : int {
  STAGE_F64 = 0,       // FP64 operator, FP64 input and output
  STAGE_MIX_IN64 = 1,  // FP32 operator reading an FP64 input (first stage, apply)
  STAGE_MIX_IN32 = 2,  // FP32 operator reading an FP32 stage input
  STAGE_FF_IN64 = 3,   // float-float operator reading an FP64 input (curved cells only)
  STAGE_FF_INFF = 4,   // float-float operator reading a float-pair stage input (curved cells only)
  N_STAGE_VARIANTS = 5
};

struct KernelEntry {
  cudaError_t (*launch)(const LaunchArgs&, int grid, cudaStream_t) = nullptr;
  int (*occupancy)(int cells_per_block) = nullptr;
  size_t (*smem)(int cells_per_block) = nullptr;
};

// Variants of the Cartesian line kernel (ew_cart.cuh): compute precision,
// input type and epilogue.
enum CartVariant : int {
  CV_F64_APPLY = 0,   // FP64: dst = M^-1 A(X)
  CV_F64_MID = 1,     // FP64 LSRK stage 1..4
  CV_F64_LAST = 2,    // FP64 LSRK stage 5 / ADER update
  CV_MIX_APPLY64 = 3, // FP32 operator on an FP64 input: dst = M^-1 A(X)
  CV_MIX_S1 = 4,      // mixed LSRK stage 1 (FP64 state in)
  CV_MIX_APPLY32 = 5, // FP32 operator on an FP32 input
  CV_MIX_MID = 6,     // mixed LSRK stages 2..4
  CV_MIX_LAST = 7,    // mixed LSRK stage 5 (FP64 state out)
  CV_MIX_UPD = 8,     // mixed ADER update u + M^-1 A(T)
  CV_MIX_S1_FF = 9,   // mixed stage 1, state held as float pairs (multi-step calls)
  CV_MIX_LAST_FF = 10,  // mixed stage 5, state left as float pairs
  CV_FF_APPLY64 = 11,   // compensated (float-float) operator on an FP64 input
  CV_FF_S1 = 12,        // compensated LSRK stage 1 (FP64 state in)
  CV_FF_MID = 13,       // compensated LSRK stages 2..4 (float-pair stage inputs)
  CV_FF_LAST = 14,      // compensated LSRK stage 5 (FP64 state out)
  CV_FF_UPD = 15,       // compensated ADER update u + M^-1 A(T), T as float pairs
  CV_FF_APPLYFF = 16,   // compensated operator on a float-pair input
  CV_FF_LAST_PAIR = 17, // compensated LSRK stage 5, state left as float pairs (multi-step calls)
  N_CART_VARIANTS = 18
};

// Launcher of the Cartesian line kernel.
struct CartEntry {
  cudaError_t (*launch)(const LaunchArgs&, int stage_x, int tma, int nb_lines, int grid,
                        cudaStream_t) = nullptr;
  int (*occupancy)(int cells_per_block, int stage_x) = nullptr;
  size_t (*smem)(int cells_per_block, int stage_x) = nullptr;
};

struct KernelTable {
  int dim = 0, np = 0, points = 0;
  int lines = 0;  // threads per cell of the Cartesian kernel: dim * np^(dim-1)
  KernelEntry stage[N_STAGE_VARIANTS][2];  // [variant][cartesian]
  CartEntry cart[N_CART_VARIANTS];
  KernelEntry ck[3][2][2];                 // [FP64 / mixed / compensated][cartesian][post]
  // the same without spectral evaluation (no degree reduction); empty below
  // degree 4, where both are the same
  KernelEntry ck_full[3][2][2];
  // upload the even-odd 1D constants of this degree to the current device
  cudaError_t (*set_constants)(const double* w, const double* D, const double* L0,
                               const double* L1) = nullptr;
};

#define EW_DECL(d, n) void kernel_table_d##d##_##n(KernelTable&);
EW_DECL(2, 2) EW_DECL(2, 3) EW_DECL(2, 4) EW_DECL(2, 5) EW_DECL(2, 6) EW_DECL(2, 7) EW_DECL(2, 8)
EW_DECL(2, 9) EW_DECL(2, 10) EW_DECL(2, 11) EW_DECL(2, 12) EW_DECL(2, 13)
EW_DECL(3, 2) EW_DECL(3, 3) EW_DECL(3, 4) EW_DECL(3, 5) EW_DECL(3, 6) EW_DECL(3, 7) EW_DECL(3, 8)
EW_DECL(3, 9) EW_DECL(3, 10) EW_DECL(3, 11) EW_DECL(3, 12) EW_DECL(3, 13)
#undef EW_DECL

}  // namespace ew
