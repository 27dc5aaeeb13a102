// ew_internal.h -- host-side pieces shared by the single-solve context
// (ew_api.cu) and the batch runtime (ew_batch.cu).
#pragma once

#include <string>

#include "../../include/exwave_gb300.h"
#include "ew_launch.h"

namespace ew {

// kernel launchers for (dim, points per direction), built once
const KernelTable& kernel_table(int dim, int np);

// Checks a mesh description; on success *cartesian tells whether every cell
// is an axis-aligned box.  On failure returns an ew_status and fills *err.
int validate_mesh(const ew_mesh_desc* m, bool* cartesian, std::string* err);

// Uploads the Cartesian kernel's 1D constants of this degree to the
// current device.
cudaError_t upload_cart_constants(int dim, int np);

// One block waiting on an mbarrier that nothing completes, giving up after
// `polls` tries and raising ERR_WAIT_TIMEOUT in *err (ew_diag.cu).
cudaError_t launch_wait_timeout(int polls, int* err, cudaStream_t stream);

// FP64 state -> interleaved float pairs (hi, lo: the exact split) in the
// same 8-byte slots; pairs may be state (in place) (ew_batch.cu).
cudaError_t launch_split_pairs(const double* state, int64_t n, void* pairs, cudaStream_t stream);

// Tuned cells per block for (dim, degree, precision); 0 when unset.
int tuned_cells_per_block(int dim, int degree, int precision);
// Tuned neighbour staging of the line kernel (0 unset, 1 lines, 2 bulk).
int tuned_staging(int dim, int degree, int precision);

// LowStorageRK45Reg2 coefficients (time_integrators.cc:243-252)
constexpr double kA21 = 970286171893. / 4311952581923.;
constexpr double kA32 = 6584761158862. / 12103376702013.;
constexpr double kA43 = 2251764453980. / 15575788980749.;
constexpr double kA54 = 26877169314380. / 34165994151039.;
constexpr double kB1 = 1153189308089. / 22510343858157.;
constexpr double kB2 = 1772645290293. / 4653164025191.;
constexpr double kB3 = -1672844663538. / 4480602732383.;
constexpr double kB4 = 2114624349019. / 3568978502595.;
constexpr double kB5 = 5198255086312. / 14908931495163.;

}  // namespace ew
