/* exwave_gb300.h -- C ABI of the GB300-native ExWave DG operator hot path.
 *
 * The library re-implements, as CUDA kernels for sm_103a, the explicit
 * upwind DG operator of ExWave (kronbichler/exwave) for the first-order
 * acoustic system (pressure p, velocity u) on FE_DGQ(k) quads and hexes,
 * the low-storage Runge-Kutta stage update around it and the ADER
 * Taylor / Cauchy-Kovalevskaya time-integral sweep.  Every entry point below
 * names the reference interface it replaces.
 *
 * Conventions shared by all calls
 *  - State vectors are FP64 device pointers in the canonical layout
 *    [cell][field][point]: fields u_0..u_{d-1}, p; points are the (k+1)^d
 *    Gauss points of the cell in lexicographic order (x fastest).  The DG
 *    solution is stored by its values at the Gauss points (collocation basis
 *    of QGauss(k+1)), so n_dofs = n_cells * (d+1) * (k+1)^d, as in the
 *    reference's FE_DGQ(k) system.
 *  - Every call returns EW_OK (0) or a negative ew_status; no exception
 *    crosses the ABI.  ew_last_error() gives a message.  Kernels run on the
 *    context's stream and return asynchronously; ew_synchronize() waits and
 *    reports device-side errors (bad neighbour index, wait time-out).
 *  - One context is used by one host thread at a time (the reference's
 *    operator mutates scratch in const methods as well).
 */
#ifndef EXWAVE_GB300_H
#define EXWAVE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EW_MAX_DEGREE 12 /* k = 1..12, as the reference instantiates */

typedef enum ew_status {
  EW_OK = 0,
  EW_ERR_INVALID = -1,     /* bad argument or inconsistent mesh */
  EW_ERR_UNSUPPORTED = -2, /* valid in the reference, not built here */
  EW_ERR_CUDA = -3,        /* CUDA runtime error */
  EW_ERR_OOM = -4,         /* device allocation failed */
  EW_ERR_DEVICE = -5,      /* a kernel raised the device error flag */
  EW_ERR_TOO_LARGE = -6    /* size above a fixed limit */
} ew_status;

typedef enum ew_precision {
  EW_PREC_FP64 = 0,     /* operator, geometry and state in FP64 */
  EW_PREC_MIXED = 1,    /* operator and geometry in FP32, state/accumulation FP64 */
  EW_PREC_MIXED_FF = 2  /* compensated: stage inputs as float pairs, the operator's
                           arithmetic and coefficients in float-float (about 44
                           bits), state FP64; equal to the FP64 path to about
                           1e-14.  Axis-aligned and curved cells, every
                           integrator, ADER and batches; the static step
                           (ew_lsrk45_step_static) returns EW_ERR_UNSUPPORTED */
} ew_precision;

typedef enum ew_boundary {
  EW_BC_SOFT_WALL = 1, /* u.n = 0 */
  EW_BC_HARD_WALL = 2, /* p = 0 */
  EW_BC_ABSORBING = 3  /* first-order absorbing condition */
} ew_boundary;

/* Mesh of one solve, the flattened equivalent of the reference's
 * MatrixFree setup (WaveEquationOperation::setup / reset_data_vectors,
 * wave_equation_operations.cc:200-250, 383-400).  Host pointers; copied to the
 * device by ew_create.
 *  vertices : [n_cells][2^dim][dim] cell vertices, deal.II lexicographic
 *             vertex order; cells are multilinear (MappingQGeneric on a flat
 *             manifold interpolates exactly this map).
 *  neighbors: [n_cells][2*dim] for face f = 2*direction + side: the index of
 *             the cell across the face, which must see it as its face f^1
 *             with the same tangential orientation; or -id for a boundary
 *             face with boundary id 1, 2 or 3.
 *  speed, density: [n_cells] material per cell (c, rho). */
typedef struct ew_mesh_desc {
  int32_t dim;
  int32_t degree;
  int64_t n_cells;
  const double* vertices;
  const int32_t* neighbors;
  const double* speed;
  const double* density;
} ew_mesh_desc;

typedef struct ew_options {
  int32_t precision;           /* ew_precision */
  int32_t use_ader_post;       /* reference parameter ADER/use_ader_post */
  int32_t spectral_evaluation; /* reference ADER/spectral_evaluation (parameters.cc:76):
                                  1 (default) degree reduction, 0 full degree throughout */
  int32_t cells_per_block;     /* 0: tuned default */
  int32_t device;              /* CUDA device ordinal */
  /* shared-memory layout of the line kernel's neighbour data (3-D degrees
   * where both are built): 0 tuned default, 1 each thread's neighbour lines
   * by per-thread asynchronous copies, 2 the neighbours' whole field arrays
   * by bulk copies */
  int32_t nb_staging;
} ew_options;

typedef struct ew_ctx ew_ctx;

/* Replaces WaveEquationOperation<dim,k>::setup (wave_equation_operations.cc:200-250)
 * and the ADER setup (276-315): validates the mesh, flattens geometry and
 * materials to the device and allocates the operator's scratch. */
int ew_create(const ew_mesh_desc* mesh, const ew_options* options, ew_ctx** ctx);
void ew_destroy(ew_ctx* ctx);

/* Message of the last failure on ctx, or of the calling thread's last failed
 * ew_create when ctx is NULL. */
const char* ew_last_error(const ew_ctx* ctx);

/* Stream for all later work of ctx (a cudaStream_t; NULL = legacy stream). */
int ew_set_stream(ew_ctx* ctx, void* stream);
int64_t ew_n_dofs(const ew_ctx* ctx);
int64_t ew_n_cells(const ew_ctx* ctx);

/* Replaces WaveEquationOperation::apply (wave_equation_operations.cc:665-685):
 * dst = M^{-1} A(src), the cell, inner-face and boundary-face terms followed
 * by the inverse mass matrix, in one kernel. */
int ew_apply(ew_ctx* ctx, const double* src, double* dst);

/* Replaces RKVectorUpdater::apply_to_subrange (time_integrators.cc:129-155):
 * not last: v2 += f1*v1; v3 = v2 + f2*v1.  last: v2 = v3 + f1*v1. */
int ew_rk_update(ew_ctx* ctx, double f1, double f2, int32_t is_last, const double* v1,
                 double* v2, double* v3);

/* Replaces LowStorageRK45Reg2::perform_time_step (time_integrators.cc:235-283):
 * five fused operator+update stages; on return vec_np holds the new state
 * and vec_n has been used as a register (its content is undefined), as in
 * the reference. */
int ew_lsrk45_step(ew_ctx* ctx, double dt, double* vec_n, double* vec_np);

/* The same step on HOST vectors, the storage of the reference's
 * perform_time_step (its LA::distributed::Vector<double> lives in host
 * memory): h_vec_n is copied to a device vector owned by the context, the
 * step runs on the context stream, and the new state is copied to h_vec_np
 * (h_vec_n is not modified unless it is h_vec_np; both may be the same
 * array).  The copies run in chunks on two internal streams: when a call's
 * input is the previous call's output, each chunk's host-to-device copy
 * starts as soon as the previous call's device-to-host copy of that chunk
 * has landed, so the two directions overlap; on axis-aligned meshes the
 * stages also run chunk by chunk beside the copies (all five as a wavefront
 * when every chunk's neighbours lie in the chunks next to it, else the
 * first and the last).  Results equal ew_lsrk45_step's bit for bit.  Host arrays should be pinned
 * (cudaHostAlloc / cudaHostRegister) for the copies to be asynchronous.
 * Returns once the work is enqueued; h_vec_np is complete after
 * ew_synchronize, or on the context stream after ew_wait_host_copies.  The
 * step itself runs on a stream of the context's own, after the work on the
 * context stream at the call; every later call on the context orders the
 * context stream after it. */
int ew_lsrk45_step_host(ew_ctx* ctx, double dt, const double* h_vec_n, double* h_vec_np);
/* Orders the context stream after the device-to-host copies of the last
 * ew_lsrk45_step_host call (an event recorded or a synchronize on the stream
 * afterwards covers them). */
int ew_wait_host_copies(ew_ctx* ctx);

/* Low-storage 2-register schemes of the reference, selected by
 * ew_lsrk_scheme: replaces LowStorageRK33Reg2 (time_integrators.cc:200-233),
 * LowStorageRK45Reg2 (:235-283, the same as ew_lsrk45_step) and
 * LowStorageRK59Reg2 (:286-364)::perform_time_step.  One fused
 * operator+update launch per stage; vec_n is used as a register, the new
 * state is left in vec_np. */
typedef enum ew_lsrk_scheme { EW_LSRK33R2 = 0, EW_LSRK45R2 = 1, EW_LSRK59R2 = 2 } ew_lsrk_scheme;
int ew_lsrk_step(ew_ctx* ctx, int32_t scheme, double dt, double* vec_n, double* vec_np);

/* y = alpha*y + (beta*x + gamma*z) over the context's n_dofs: the vector
 * operations of the reference's composed integrators (deal.II Vector::add
 * with alpha = 1, Vector::sadd with gamma = 0, assignment with alpha = 0 and
 * beta = 1), used by ExplicitEuler, ClassRK4, LowStorageRK45Reg3 and SSPRK
 * (time_integrators.cc:24-31, 66-102, 366-427, 440-478).  A NULL x or z
 * drops its term; alpha == 0 does not read y.  All device vectors. */
int ew_vec_update(ew_ctx* ctx, double alpha, double* y, double beta, const double* x, double gamma,
                  const double* z);

/* n_steps LSRK45 steps in one call: the reference's time loop
 * (explicit_wave.cc:779-799) calling perform_time_step and swapping the two
 * vectors n_steps times.  On entry vec_n holds u^n; on return vec_np holds
 * u^{n+n_steps} and vec_n is undefined.  With mixed precision on Cartesian
 * meshes the state between two steps of the call is kept as an unevaluated
 * float pair (hi + lo, about 48 significant bits) instead of being rounded
 * to FP64, so the first stage of each following step reads it pre-split;
 * the final state is FP64. */
int ew_lsrk45_steps(ew_ctx* ctx, double dt, int64_t n_steps, double* vec_n, double* vec_np);

/* Receivers: point evaluation of the solution, the data a time_step_analysis
 * hook (utilities.h:136-142) records at fixed points.  ew_set_receivers
 * locates n points (host array, n x dim, physical coordinates) once: the
 * containing cell and the reference coordinates (Newton's method on the
 * multilinear map), then the Lagrange weights of the Gauss-point basis.
 * EW_ERR_INVALID names the first point outside the mesh.  Replaces any
 * earlier set. */
int ew_set_receivers(ew_ctx* ctx, int32_t n, const double* points);

/* ADER in its ADERADCONFULL form: WaveEquationOperationADERADCONFULL::apply_ader
 * (wave_equation_operations.cc:689-735), the Taylor series of the time
 * integral built from k+1 applications of the full DG operator, followed by
 * the update of ArbitraryHighOrderDG::perform_time_step (time_integrators.cc:37-50).
 * vec_n is not modified; two FP64 work vectors are allocated on first use. */
int ew_aderadconfull_step(ew_ctx* ctx, double dt, const double* vec_n, double* vec_np);

/* Every field (u_0..u_{d-1}, p) of a device state at the receivers into the
 * device array out (n x (dim+1), receiver-major), on the context's stream. */
int ew_sample_receivers(ew_ctx* ctx, const double* state, double* out);

/* The same LSRK45 step as ew_lsrk45_step, for callers that cannot have the
 * library allocate device memory: it has no counterpart in the reference.
 * Code that runs the step inside an application which owns all device
 * memory through its own pool or a fixed budget, or inside a
 * latency-sensitive loop, cannot use cudaMalloc there (it synchronises the
 * device and fails when the pool holds the memory).  This entry point keeps
 * its stage scratch in one static device array of EW_STATIC_SCRATCH_BYTES
 * (64 MiB) that every GPU loading the library holds until exit, and calls no
 * allocator.  The context itself still allocates its own integrator scratch
 * once, in ew_create, like every context; what this entry point adds is a
 * step that calls no allocator and uses the static array in place of the
 * context's buffers.  Limit: n_dofs <= EW_STATIC_SCRATCH_MAX_DOFS, larger contexts
 * get EW_ERR_TOO_LARGE.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  All calls on a device share the
 * array and it keeps the last call's contents (every stage writes the
 * scratch it later reads, so nothing has to start at zero): calls that
 * overlap on the GPU race. */
#define EW_STATIC_SCRATCH_BYTES (64ll << 20)
#define EW_STATIC_SCRATCH_MAX_DOFS ((EW_STATIC_SCRATCH_BYTES / 8) - 64)
int ew_lsrk45_step_static(ew_ctx* ctx, double dt, double* vec_n, double* vec_np);

/* Replaces WaveEquationOperationADER::apply_ader (wave_equation_operations.cc:1346-1381):
 * T = Taylor time integral of src over [0,dt]; dst = -M^{-1} A(T). */
int ew_apply_ader(ew_ctx* ctx, double dt, const double* src, double* dst);

/* Replaces ArbitraryHighOrderDG::perform_time_step (time_integrators.cc:37-50):
 * vec_np = vec_n - apply_ader(vec_n), fused into the second ADER kernel. */
int ew_ader_step(ew_ctx* ctx, double dt, const double* vec_n, double* vec_np);

/* Physical coordinates of all Gauss points, device pointer [cell][point][dim]
 * (what FEEvaluation::quadrature_point gives the reference's
 * project_initial_field, wave_equation_operations.cc:902-935). */
int ew_quadrature_points(ew_ctx* ctx, double* xyz);

/* Replaces project_initial_field for the vibrating-membrane field: a sum of
 * modes p = sum A_m cos(w_m t) prod_d sin(k_md pi x_d) with the matching
 * velocity (c = rho = 1; input_parameters.h:95-128 is the one-mode case).
 * amp[n_modes], kvec[n_modes][3] are host arrays; u is a device vector. */
int ew_project_membrane(ew_ctx* ctx, int32_t n_modes, const double* amp, const int32_t* kvec,
                        double t, double* u);

/* Gaussian pressure pulse p = amp*exp(-|x-x0|^2/(2 width^2)), u = 0. */
int ew_project_gaussian(ew_ctx* ctx, const double* x0, double width, double amp, double* u);

/* L2 errors against the membrane solution with QGauss(k+2) on the mapped
 * cells (explicit_wave.cc:439-496): out[0] = |p_h - p|, out[1] = |u_h - u|,
 * out[2] = |p|.  Synchronises. */
int ew_l2_errors_membrane(ew_ctx* ctx, const double* u, int32_t n_modes, const double* amp,
                          const int32_t* kvec, double t, double out[3]);

/* "error p post": the post-processed pressure p* of degree k+1 per cell
 * (WaveEquationOperation::compute_post_pressure,
 * wave_equation_operations.cc:784-848: (grad phi, grad p*) =
 * (grad phi, -rho du/dt) with QGauss(k+2), du/dt = M^-1 A(u), one value
 * constrained, CG to 1e-11, then shifted to the mean of p_h) and its L2
 * error against the membrane pressure with QGauss(k+3)
 * (explicit_wave.cc:476-484).  FP64 throughout except du/dt and the
 * density, which a mixed context holds in FP32.  Synchronises. */
int ew_l2_error_post_membrane(ew_ctx* ctx, const double* state, int32_t n_modes,
                              const double* amps, const int32_t* kvecs, double t, double* out);

/* L2 norm of the difference of two states with QGauss(k+2) (pressure,
 * velocity); used for FP64-vs-mixed comparisons.  Synchronises. */
int ew_l2_difference(ew_ctx* ctx, const double* a, const double* b, double out[2]);

/* Structured mesh generator: the reference's input_geometry_description
 * (input_parameters.h:60-88): subdivided_hyper_cube(n_intervals) of [0,1]^dim,
 * a vertex transform, then n_refinements global refinements with a flat
 * manifold (new vertices on the multilinear map of each coarse cell).
 * Cells are numbered lexicographically on the fine grid, x fastest.
 *  transform 0: the reference's x_0 += f prod_d sin(pi x_d) (input_parameters.h:42-50)
 *  transform 1: every coordinate x_i += f prod_d sin(2 pi x_d)
 *  boundary_ids[2*d + s]: id of the domain face x_d = s (s = 0, 1). */
typedef struct ew_hypercube_desc {
  int32_t dim;
  int32_t n_intervals;
  int32_t n_refinements;
  int32_t transform;
  double transform_factor;
  int32_t boundary_ids[6];
} ew_hypercube_desc;

int64_t ew_hypercube_n_cells(const ew_hypercube_desc* desc);

/* Fills host arrays vertices[n_cells][2^dim][dim] and
 * neighbors[n_cells][2*dim] in the ew_mesh_desc conventions. */
int ew_hypercube_mesh(const ew_hypercube_desc* desc, double* vertices, int32_t* neighbors);

/* Change of nodal basis per cell, on the host, for adapters whose vectors
 * hold Q_k by its values at other 1-D support points.  The reference's
 * FE_DGQ(k) (explicit_wave.cc:162) uses k+1 equidistant points on [0,1];
 * FEEvaluation interpolates those coefficients to QGauss(k+1) before the
 * operator (wave_equation_operations.cc:411-419).  This library stores the
 * Gauss-point values directly.  src and dst: host arrays
 * [n_cells][n_fields][(k+1)^dim], points lexicographic (x fastest); `nodes`
 * holds the k+1 distinct 1-D support points.  Both directions are exact
 * (the same Q_k polynomial).  The caller still maps its own DoF numbering
 * to this per-cell order.
 *  ew_nodal_to_gauss: values at `nodes` -> values at the Gauss points
 *  ew_gauss_to_nodal: the inverse */
int ew_nodal_to_gauss(int32_t dim, int32_t degree, int64_t n_cells, int32_t n_fields,
                      const double* nodes, const double* src, double* dst);
int ew_gauss_to_nodal(int32_t dim, int32_t degree, int64_t n_cells, int32_t n_fields,
                      const double* nodes, const double* src, double* dst);

/* ---------------------------------------------------------------- batches
 * Many independent solves (uneven degree, mesh size, material, source) in
 * one device-resident batch: each step advances every unfinished solve by
 * one LSRK45 step with one persistent launch per (dimension, degree) group
 * and stage over a work list of cell blocks; the per-step launch sequence is
 * captured as a CUDA graph.  Admission is bounded by an HBM budget (device
 * arena allocated once).  No reference counterpart: the reference advances
 * one mesh per MPI job. */
typedef struct ew_batch ew_batch;

typedef struct ew_batch_options {
  int32_t precision;        /* ew_precision */
  int32_t device;
  int64_t hbm_budget_bytes; /* arena size */
  int32_t max_solves;
  int32_t use_graphs;       /* 1: capture each step as a CUDA graph */
  /* 1: ew_batch_step may take a solve past its n_steps; the extra steps are
   * computed but neither sampled nor counted, so that a serving tick of many
   * steps is not cut short by the solve with the fewest steps left (its state
   * is then no longer the one at n_steps) */
  int32_t allow_overrun;
  int32_t reserved;
  /* a solve whose receiver samples become non-finite, or larger in magnitude
   * than this (when > 0), is marked diverged: ew_batch_diverged reports it */
  double blowup_limit;
} ew_batch_options;

/* Ricker point source added to the pressure equation:
 * amplitude * (1 - 2 pi^2 f0^2 s^2) exp(-pi^2 f0^2 s^2), s = t - delay. */
typedef struct ew_source_desc {
  double position[3];
  double frequency;
  double delay;
  double amplitude;
} ew_source_desc;

typedef struct ew_solve_desc {
  ew_mesh_desc mesh;        /* Cartesian cells */
  double dt;
  int64_t n_steps;          /* the solve ends after n_steps LSRK45 steps */
  int32_t n_sources;        /* 0 or 1 */
  ew_source_desc source;
  int32_t n_receivers;      /* pressure sampled after every step */
  const double* receivers;  /* host [n_receivers][dim] */
} ew_solve_desc;

int ew_batch_create(const ew_batch_options* options, ew_batch** batch);
void ew_batch_destroy(ew_batch* batch);
const char* ew_batch_last_error(const ew_batch* batch);
/* Device bytes a solve would take from the arena. */
int64_t ew_batch_solve_bytes(const ew_batch* batch, const ew_solve_desc* solve);
int64_t ew_batch_bytes_free(const ew_batch* batch);
/* Admits a solve (zero initial state); EW_ERR_OOM when the arena cannot hold it. */
int ew_batch_add(ew_batch* batch, const ew_solve_desc* solve, int32_t* id);
/* Releases a solve's memory. */
int ew_batch_remove(ew_batch* batch, int32_t id);
/* Copies a caller's device FP64 state (canonical layout) into a solve. */
int ew_batch_set_state(ew_batch* batch, int32_t id, const double* state);
/* Copies a solve's current FP64 state to a caller's device buffer. */
int ew_batch_get_state(ew_batch* batch, int32_t id, double* state);
/* Advances every unfinished solve by n_steps (at most the smallest number
 * of steps any unfinished solve has left, unless allow_overrun is set). */
int ew_batch_step(ew_batch* batch, int32_t n_steps);
int ew_batch_info(const ew_batch* batch, int32_t id, int64_t* steps_done, int64_t* n_steps);
/* Ids of the solves marked diverged so far (at most capacity), after the
 * batch's stream finishes; the caller removes them.  The analogue of the
 * reference's blow-up test (explicit_wave.cc:498-507), per solve and on the
 * device: the receiver samples of every step are checked. */
int ew_batch_diverged(ew_batch* batch, int32_t* ids, int32_t capacity, int32_t* count);
/* Receiver samples [first, first + count) of a solve into host out[count][n_receivers]. */
int ew_batch_receivers(ew_batch* batch, int32_t id, int64_t first, int64_t count, double* out);
int ew_batch_set_stream(ew_batch* batch, void* stream);
int ew_batch_synchronize(ew_batch* batch);
int64_t ew_batch_kernel_launches(const ew_batch* batch);

/* Tuning table consulted by ew_create (when options->cells_per_block is 0)
 * and by the batch runtime: cells per thread block of the operator kernel
 * for (dim, degree, precision); 0 restores the built-in default.  Written by
 * the autotuner (exwave_gb300/autotune.py).  No reference counterpart. */
int ew_tune_set(int32_t dim, int32_t degree, int32_t precision, int32_t cells_per_block);
int32_t ew_tune_get(int32_t dim, int32_t degree, int32_t precision);
/* The same table's neighbour staging (ew_options.nb_staging; 0 restores the
 * built-in choice). */
int ew_tune_set_staging(int32_t dim, int32_t degree, int32_t precision, int32_t nb_staging);
int32_t ew_tune_get_staging(int32_t dim, int32_t degree, int32_t precision);

/* Waits for the context's stream and reports a raised device error flag. */
int ew_synchronize(ew_ctx* ctx);

/* Diagnostic of the failure path of the staged kernels (no reference
 * counterpart): one block waits on an mbarrier that nothing completes, with
 * the same bounded wait the kernels use but a limit of `polls` tries; it
 * gives up, raises the time-out flag and returns, with no copy in flight.
 * Returns what ew_synchronize then reports: EW_ERR_DEVICE (flag cleared), and
 * the context stays usable. */
int ew_check_wait_timeout(ew_ctx* ctx, int32_t polls);

/* Number of kernels this library has launched on ctx so far. */
int64_t ew_kernel_launches(const ew_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* EXWAVE_GB300_H */
