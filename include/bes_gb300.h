/*
 * bes_gb300 — GB300-native (sm_103a) steady residual/update path of the Basic Euler Solver
 * (joel-ho/BES).  Plain C ABI: opaque handle, plain pointers and sizes, int status codes
 * (0 = ok), no exceptions across the boundary.  All arrays passed in are borrowed and copied;
 * the library owns its device memory.  One context is used by one host thread at a time and
 * runs on its own CUDA stream.
 *
 * Numbering: every array exchanged through this interface is in the REFERENCE numbering, the
 * numbering the reference assigns when it reads the same Gmsh file (cells in file order; faces
 * in creation order: boundary triangles first, then the tetrahedra's new faces).  Internally the
 * library renumbers cells (reverse Cuthill-McKee) and faces (interior faces sorted by owner,
 * then slip-wall faces, then freestream faces).
 *
 * Layouts: a cell state is [n_cells][5] (rho, rho u, rho v, rho w, rho E); gradients are
 * [n_cells][5][3]; limiters [n_cells][5]; face fluxes [n_faces][5] per unit area.
 */
#ifndef BES_GB300_H
#define BES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define BES_OK 0
#define BES_ERR_INVALID 1     /* bad argument or size */
#define BES_ERR_CUDA 2        /* CUDA runtime error or no CUDA device */
#define BES_ERR_NAN 3         /* NaN in a face flux (the reference exits, src/SolverExplicit.cpp:312-322) */
#define BES_ERR_MESH 4        /* mesh cannot be used (missing boundary triangle, unknown tag, ...) */
#define BES_ERR_CONFIG 5      /* .besi option error (unknown key or value, src/Config.cpp:415-418) */
#define BES_ERR_UNSUPPORTED 6 /* option combination not implemented */
#define BES_ERR_TIMEOUT 7     /* a bounded device wait gave up */

/* boundary tags of the mesh arrays (the Gmsh physical names SLIP_WALL / FREESTREAM,
 * src/Options.cpp:22-26) */
#define BES_TAG_SLIP_WALL 1
#define BES_TAG_FREESTREAM 2

/* Mesh as read from a Gmsh 2.2 file: nodes, the boundary faces in file order, then the cells
 * in file order.  All ids 0-based.  3-D (dim 0 or 3): boundary triangles and tetrahedra.
 * 2-D (dim 2, Mesh::readGmsh's nDim from the physical names, src/Mesh.cpp:170-183): boundary
 * lines [n_btris][2] and triangles [n_tets][3], counter-clockwise; z is ignored. */
typedef struct {
  int64_t n_nodes;
  const double* nodes;   /* [n_nodes][3] */
  int64_t n_btris;
  const int64_t* btris;  /* [n_btris][3] (2-D: [n_btris][2]) */
  const int32_t* btags;  /* [n_btris] BES_TAG_* */
  int64_t n_tets;
  const int64_t* tets;   /* [n_tets][4] positively oriented (2-D: [n_tets][3]) */
  int32_t dim;           /* 0 or 3: tetrahedra; 2: triangles */
} bes_mesh_arrays;

static inline int bes_mesh_dim(const bes_mesh_arrays* m) { return m->dim == 2 ? 2 : 3; }

/* Options: the .besi keys of the reference (src/Config.cpp:73-422) plus additive keys. */
typedef struct {
  int32_t solver_type;            /* SOLVER_TYPE: 0 EXPLICIT, 1 IMPLICIT */
  int32_t local_time_step;        /* LOCAL_TIME_STEP: 1 YES, 0 NO (default NO) */
  int32_t n_stage;                /* MULTI_TIME_STEP_OPTIONS: stage count (default 4) */
  int32_t muscl_face_vector;      /* 0: the reference's lookup (quirk Q13, default); 1: exact */
  double stage_coeff[8];          /* MULTI_TIME_STEP_OPTIONS coefficients */
  double courant_num;             /* COURANT_NUM (default 2.0) */
  double adaptive_courant_num_max;      /* ADAPTIVE_COURANT_NUM_MAX (default 0) */
  double adaptive_courant_num_exponent[2]; /* ADAPTIVE_COURANT_NUM_EXPONENT (default 1, 1) */
  double venkatakrishnan_factor;  /* VENKATAKRISHNAN_FACTOR (default 5) */
  double harten_correction_limit; /* HARTEN_CORRECTION_LIMIT (default 0.05) */
  double gas_constant;            /* GAS_CONSTANT (default 287) */
  double specific_heat_ratio;     /* SPECIFIC_HEAT_RATIO (default 1.4) */
  double freestream_mach[3];      /* FREESTREAM_MACH */
  int32_t number_of_time_step;    /* NUMBER_OF_TIME_STEP */
  int32_t linear_solver;          /* 0 block-Jacobi GMRES, 1 block-ILU(0) GMRES (colour order),
                                     2 block-ILU(0) GMRES (RCM order, level scheduled) */
  int32_t linear_solver_max_iter; /* LINEAR_SOLVER_MAX_ITER (default 1000) */
  int32_t gmres_restart;          /* GMRES_RESTART (additive, default 30) */
  double linear_solver_tol;       /* LINEAR_SOLVER_ABS_TOL: relative to |b| (default 1e-7) */
  int32_t jacobian_repeat;        /* times each Jacobian block is added (Q9); 0, the default:
                                     once per conserved variable of the mesh, 5 in 3-D and 4
                                     in 2-D, as the reference (src/SolverImplicit.cpp:425-502) */
  int32_t precision;              /* PRECISION (additive): 0 FP64, 1 FP32 linear solve,
                                     2 FP32 linear solve with the matrix and factors stored
                                     as FP16 blocks with a power-of-two scale per block and
                                     the Krylov basis stored in FP16 */
  int32_t cfl_ramp_steps;         /* CFL_RAMP (additive): steps of a geometric CFL ramp, 0 off */
  int32_t freestream_ramp;        /* FREESTREAM_RAMP: steps over which the freestream velocity
                                     ramps up (src/Config.cpp:688-706), 0 off */
  double cfl_ramp_start, cfl_ramp_end;
  double freestream_ramp_start_frac;  /* FREESTREAM_RAMP_START_FRAC (default 0.5) */
  int32_t sweep_kernel;           /* SWEEP_KERNEL (additive): block-ILU(0) colour sweeps as
                                     0 the autotuner's choice (timed on the first step's
                                     system, see bes_tuning), 1 one launch per colour, 2 one
                                     persistent launch per sweep, 3 one launch per colour
                                     with every load of a row issued first (precision 2) */
  int32_t reserved_i;
  double reserved[2];
} bes_options;

typedef struct bes_ctx bes_ctx;

/* Default options (Config::setDefaultValues_, src/Config.cpp:73-114). */
void bes_options_default(bes_options* opt);

/* Parse a .besi file (replaces Config::initialize, src/Config.cpp:116-453): same keys, same
 * strictness (unknown key -> BES_ERR_CONFIG).  mesh_path receives MESH_FILE. */
int bes_options_from_besi(const char* besi_path, bes_options* opt, char* mesh_path,
                          size_t mesh_path_cap, char* err, size_t err_cap);

/* Read a Gmsh 2.2 ASCII mesh (replaces Mesh::readGmsh, src/Mesh.cpp:95-558).  Arrays are
 * allocated by the library and freed with bes_mesh_free. */
int bes_mesh_read_gmsh(const char* path, bes_mesh_arrays* out, char* err, size_t err_cap);
void bes_mesh_free(bes_mesh_arrays* mesh);

/* Create a context on the current CUDA device: build the reference-semantics mesh (face
 * discovery, geometry, quirks), renumber, upload.  Replaces main()'s Config/Mesh/Gas/Solver
 * construction (src/BES.cpp:86-106) and Solver::initialize (include/Solver.hpp:70). */
int bes_create(const bes_mesh_arrays* mesh, const bes_options* opt, bes_ctx** out);
void bes_destroy(bes_ctx* ctx);
const char* bes_last_error(const bes_ctx* ctx);
int bes_sizes(const bes_ctx* ctx, int64_t* n_cells, int64_t* n_faces);

/* Solver::setUniversalInitialCondition with the freestream primitives (include/Solver.hpp:71). */
int bes_set_freestream_state(bes_ctx* ctx);
int bes_set_state(bes_ctx* ctx, const double* U);  /* [n_cond][n_cells][5] */
int bes_get_state(bes_ctx* ctx, double* U);        /* [n_cond][n_cells][5] */

/* Operators at the current state (the reference operator classes):
 *   TimeStepCalculator::computeAllTimeStep + getTimeStep (TimeStepCalculator.hpp:43-46)
 *   Gradient::computeGradient + getGradient (Gradient.hpp:46-49)
 *   Limiter::computeLimiterTerm + getLimiterValue (Limiter.hpp:47-51)
 *   the face loop's MUSCL states and Flux_<double>::computeFlux (Solver.cpp:69-121,
 *   Flux.hpp:43-46) and the residual sum R (SolverExplicit.cpp:326-340).
 * Any output pointer may be NULL. */
int bes_compute_operators(bes_ctx* ctx, double cfl, double* dt, double* grad, double* limiter,
                          double* face_UL, double* face_UR, double* face_flux, double* residual);

/* n explicit multi-step iterations (SolverExplicit::timeStep_, src/SolverExplicit.cpp:259-393).
 * history (may be NULL): [n][n_cond][10] = L2 and max norm per variable of the last stage's R
 * (zeros for a frozen condition). */
int bes_explicit_iterations(bes_ctx* ctx, int64_t n, double* history);

/* (batched contexts: history [n][n_cond][19], see bes_create_batch)
 * n implicit pseudo-time steps (SolverImplicit::timeStep_, src/SolverImplicit.cpp:293-345):
 * local/global dt at the step's CFL, second-order residual, first-order Jacobians assembled
 * into the 5x5-block system (each block added jacobian_repeat times, Q9), right-preconditioned
 * GMRES(gmres_restart) to linear_solver_tol relative with a block-Jacobi (linear_solver 0),
 * colour-ordered block-ILU(0) (1) or RCM-ordered level-scheduled block-ILU(0) (2)
 * preconditioner, in FP64 (precision 0) or FP32
 * (precision 1, defect correction: residual, update and norms stay FP64; precision 2 also
 * reads the matrix and the factors from 16-bit block-scaled copies and keeps the Krylov basis
 * in FP16), the update, and the
 * CFL control (adaptive as adaptCourantNum_, src/SolverImplicit.cpp:530-550, or the additive
 * geometric ramp).  One step of every active condition is one CUDA graph launch: the GMRES
 * iteration (Arnoldi steps, Givens rotations, restarts, convergence test) runs on the device
 * inside the graph's conditional nodes, and the host synchronises once per step.
 * history (may be NULL): [n][19] = L2[5] and max[5] of the Dt/V-scaled
 * right-hand side (the max is what the reference logs, Q10), CFL used, CFL after the step,
 * linear iterations, final relative linear residual, L2[5] of the unscaled residual
 * R = sum(+-F A) (the convergence measure).  A frozen condition (bes_set_active) does not
 * step; its history rows are zeros.  Returns BES_ERR_TIMEOUT when a linear solve was stopped
 * by its restart-cycle limit (bes_set_linear_guard); the step is applied and the context stays
 * usable. */
int bes_implicit_steps(bes_ctx* ctx, int64_t n, double* history);

/* Implicit-path statistics: out[0] steps taken, out[1] host synchronisations inside
 * bes_implicit_steps (one per step), out[2] Arnoldi steps and out[3] restart cycles the device
 * ran (each counted once per batched launch, whatever the number of conditions).  out [4]. */
int bes_implicit_stats(const bes_ctx* ctx, int64_t* out);

/* The implicit path's tuning report: for each tuned choice, the candidates with their measured
 * device times and the one taken (one line each).  Empty until the first implicit step. */
int bes_tuning(const bes_ctx* ctx, char* buf, size_t cap);

/* Limit of restart cycles per linear solve (0: linear_solver_max_iter + 1, more than a solve
 * can take).  A solve that reaches the limit stops with its current iterate and the step
 * returns BES_ERR_TIMEOUT.  The device loop over restart cycles ends by construction; this
 * bound is its guard and lets a caller cap the work of one step. */
int bes_set_linear_guard(bes_ctx* ctx, int32_t max_cycles);

/* Assemble (without solving or updating) the implicit system at the current state and CFL
 * (SolverImplicit::computeFaceFluxes_ and the CoefficientMatrix, src/SolverImplicit.cpp:358-507).
 * rhs [n_cells][5]; blocks [n_blocks][5][5] row-major in the reference's block order (row by
 * cell, diagonal block first, then neighbours in local face order,
 * src/CoefficientMatrix.cpp:141-160).  Pass NULL arrays to query n_blocks. */
int bes_implicit_assemble(bes_ctx* ctx, double cfl, double* rhs, double* blocks, int64_t* n_blocks);

/* Device timing of the implicit path by kernel category (diagnostics for benchmarking).
 * enable 1 turns timing on (the step graph then reads the GPU's nanosecond timer before and
 * after every category's work inside the graph), 0 off.  Returns (and resets) the accumulated
 * milliseconds and launch-group counts since the previous call: ms_out / counts_out [8] =
 * residual (cell sweep + face fluxes), Jacobians, assembly, ILU factorisation, preconditioner
 * application, matrix-vector products, Gram-Schmidt and GMRES control, state update.  A
 * batched launch (all conditions of a batch) counts once. */
int bes_profile(bes_ctx* ctx, int32_t enable, double* ms_out, int64_t* counts_out);

/* The block-ILU(0) factorisation order (reference cell ids, colour by colour). */
int bes_ilu_order(bes_ctx* ctx, int64_t* order);

/* Per-face fluxes and first-order Jacobians for n independent faces (unit-test entry point;
 * FluxRoe_/FluxSlipWall_/FluxFreestream_ ::computeFlux and FluxJacobianWrapper_::computeJacobian,
 * src/FluxJacobianWrapper.tpp:32-82).  kind 0 Roe, 1 slip wall, 2 freestream (UR unused; the
 * context's freestream).  Host arrays: UL, UR [n][5], nhat [n][3]; F [n][5]; JL, JR [n][5][5]
 * row-major (JR only for Roe), JL/JR may be NULL. */
int bes_flux_batch(bes_ctx* ctx, int32_t kind, int64_t n, const double* UL, const double* UR,
                   const double* nhat, double* F, double* JL, double* JR);

/* Asynchronous form of bes_explicit_iterations for pipelines and benchmarks: enqueue n
 * iterations (CUDA graph launches) on the context's stream and return without waiting.
 * bes_synchronize waits and reports a NaN flux or CUDA error of the enqueued work;
 * bes_stream returns the context's cudaStream_t; bes_last_kernel_times gives the device
 * milliseconds of the most recent iteration's kernels (ms_out [4]: cell sweep, face flux,
 * update, sum), read from event pairs captured around every kernel. */
int bes_explicit_enqueue(bes_ctx* ctx, int64_t n);
int bes_synchronize(bes_ctx* ctx);
void* bes_stream(bes_ctx* ctx);
int bes_last_kernel_times(bes_ctx* ctx, double* ms_out);

/* Residual norms without any device allocation.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc (a framework whose caching allocator already holds
 * the device memory, or a latency-critical loop where cudaMalloc/cudaFree would synchronise
 * the device).  Computes, on `stream` (NULL = default stream), the L2 and max norm per variable
 * of residual [n_cells][5] (device memory, e.g. as laid out by bes_compute_operators) into
 * norms [10] (device memory: L2[5], then max[5]), with the block reduction of the explicit
 * iteration.  Its scratch is a fixed 1.25 MiB array in device memory owned by the library
 * (held on every GPU that loads the library until the process exits), so n_cells is limited to
 * 4,194,304; larger sizes return BES_ERR_INVALID with a message in err.  The first call in
 * each CUDA context (the device's primary context, or a context the caller made current with
 * the driver API) looks up the array's device address in that context (cudaGetSymbolAddress)
 * and keeps it for the process; make that first call before any stream capture, and do not
 * call this entry point again after resetting the device.  The scratch is shared by all calls:
 * calls that overlap on the GPU race.  Returns after enqueueing (does not synchronise). */
int bes_residual_norms_static(const double* residual, int64_t n_cells, double* norms,
                              void* stream, char* err, size_t err_cap);

/* Integrated slip-wall pressure force F = sum over slip-wall faces of p S (owner-cell
 * pressure, dimensional face normal S, non-dimensional units), the quantity behind the
 * reference's slip-wall output (src/SolutionSnapshot.cpp:268-309).  force [3]. */
int bes_wall_force(bes_ctx* ctx, double* force);  /* force [n_cond][3] */

/* ---- Batched freestream sweep ----------------------------------------------------------
 * n_cond freestream conditions on one mesh in one context (no reference counterpart: the
 * reference runs one condition per process).  The mesh, geometry and graphs are shared; every
 * per-condition array holds n_cond copies, every explicit kernel takes the condition from its
 * grid's y index, and one graph launch advances all conditions by one iteration.  State
 * arrays are [n_cond][n_cells][5], histories [n][n_cond][10] (explicit) or [n][n_cond][19]
 * (implicit), wall forces [n_cond][3].  The implicit solver advances all active conditions
 * together (at most 256): each condition keeps its own state, CFL controller, freestream and
 * Krylov side (basis, vectors, GMRES state, and with precision 2 its 16-bit matrix and factor
 * copies); the residual, preconditioner, matrix-vector and Gram-Schmidt kernels take every
 * condition in one launch, and the assembly and factorisation run condition by condition
 * (with precision 2 through one shared FP32 scratch).  Each condition's result is bit for bit
 * that of a context created for it alone.  bes_compute_operators, bes_implicit_assemble and
 * bes_solve need n_cond = 1; bes_write writes condition 0; bes_sweep_run drives the explicit
 * solver.  mach [n_cond][3] replaces FREESTREAM_MACH. */
int bes_create_batch(const bes_mesh_arrays* mesh, const bes_options* opt, int32_t n_cond,
                     const double* mach, bes_ctx** out);
int bes_conditions(const bes_ctx* ctx, int32_t* n_cond);

/* Freeze (0) or run (1) each condition, active [n_cond]: a frozen condition's kernels return
 * at once and its state is carried over unchanged. */
int bes_set_active(bes_ctx* ctx, const int32_t* active);

/* Replace condition `cond` of a context by a new one: freestream Mach vector mach [3] (NULL:
 * keep the condition's), state U [n_cells][5] in reference numbering (NULL: the step-0
 * freestream state); the condition is made active and, in an implicit context, its CFL
 * control and step counters (CFL ramp, freestream ramp) restart at step 0.  Lets a sweep keep
 * every slot of a batch busy: a converged condition's slot takes the next one. */
int bes_set_condition(bes_ctx* ctx, int32_t cond, const double* mach, const double* U);

/* Solve n conditions to convergence with the implicit solver, through the context's slots (a
 * batched implicit context): each slot takes a condition of the queue (bes_set_condition with
 * mach [n][3] and, if U0 is not NULL, the initial state U0 [n][n_cells][5] in reference
 * numbering, e.g. a learned warm start; else the freestream), all slots step together, and a
 * slot whose condition is finished takes the next one.  A condition is finished when its
 * residual L2 (R = sum(+-F A), all five variables) is <= target[q] (if target is not NULL and
 * target[q] > 0), else <= drop times its first step's residual; or when it is not finite; or
 * after max_steps steps.  Per condition (each output may be NULL): steps [n], final_res [n]
 * its last residual relative to its first, force [n][3] the slip-wall pressure force of its
 * final state (bes_wall_force), U_out [n][n_cells][5] its final state, seconds [n] wall time
 * from its start to its finish.  No counterpart in the reference, which solves one condition
 * per process (src/BES.cpp:94-111). */
int bes_implicit_sweep(bes_ctx* ctx, int32_t n, const double* mach, const double* U0,
                       const double* target, double drop, int64_t max_steps, int64_t* steps,
                       double* final_res, double* force, double* U_out, double* seconds);

/* Run every condition until its residual L2 (all five variables, relative to its first
 * iteration of this call) drops by `drop`, or max_iter iterations.  Convergence is checked
 * every check_every iterations; converged conditions are frozen from then on.  iters [n_cond]
 * receives the iteration at which each condition met the drop (max_iter if it did not),
 * final_drop [n_cond] its last relative residual.  All conditions are active again on
 * return.  Either output may be NULL. */
int bes_sweep_run(bes_ctx* ctx, int64_t max_iter, double drop, int64_t check_every,
                  int64_t* iters, double* final_drop);

/* ---- Learned warm start --------------------------------------------------------------------
 * No counterpart in the reference, which always starts from the freestream
 * (Solver::setUniversalInitialCondition, include/Solver.hpp:71).  A coordinate MLP on the
 * context's mesh (cell centroid -> 16 Fourier features per axis, 4 FiLM-conditioned layers of
 * width 256 with SiLU, 5 outputs relative to the freestream) predicts the converged state for
 * a freestream Mach vector.  It is trained on the GPU from solutions the solver produced, with
 * BF16 tensor-core GEMMs, FP32 accumulation and AdamW on FP32 master weights; the solver then
 * converges from the prediction (the freestream stays the fallback).  Parameters are one flat
 * FP32 vector in the order of oracle/mlp_oracle.py layout(). */
typedef struct bes_mlp bes_mlp;
int bes_mlp_create(const bes_ctx* ctx, uint64_t seed, bes_mlp** out);
void bes_mlp_destroy(bes_mlp* mlp);
const char* bes_mlp_last_error(const bes_mlp* mlp);

/* Train for `steps` AdamW steps of `batch` (cell, sample) rows drawn from n_samples solutions
 * U [n_samples][n_cells][5] (reference numbering) at Mach vectors mach [n_samples][3].  The
 * condition and output normalisation are taken from these samples.  loss [steps] may be NULL.
 * batch: a multiple of 128. */
int bes_mlp_train(bes_mlp* mlp, int32_t n_samples, const double* mach, const double* U,
                  int64_t steps, int32_t batch, double lr, double weight_decay, uint64_t seed,
                  double* loss);

/* Predicted states U [n][n_cells][5] for Mach vectors mach [n][3]. */
int bes_mlp_infer(bes_mlp* mlp, int32_t n, const double* mach, double* U);

/* Set every condition of ctx to its predicted state; a condition whose prediction has a cell
 * with rho <= 0 or p <= 0 gets the freestream instead.  used [n_cond] (may be NULL): 1 where
 * the prediction was used.  Resets the context's step counters as bes_set_freestream_state. */
int bes_mlp_init_state(bes_mlp* mlp, bes_ctx* ctx, int32_t* used);

/* Checks and inspection: the flat FP32 parameters (get and/or set; n_params receives the
 * count), the scaled centroids xn [n_cells][3], one forward + backward on given rows
 * (cells [n_rows], normalised conditions [n_rows][3], normalised targets [n_rows][5];
 * n_rows a multiple of 128) returning the loss, the gradient [n_params] and the outputs
 * [n_rows][5], one AdamW step with a given gradient, and the normalisation
 * out [11] = condition mean [3], std [3], output scale [5]. */
int bes_mlp_params(bes_mlp* mlp, float* get, const float* set, int64_t* n_params);
int bes_mlp_features(bes_mlp* mlp, float* xn);
int bes_mlp_loss_grad(bes_mlp* mlp, int32_t n_rows, const int64_t* cells, const double* cond,
                      const double* targets, double* loss, float* grad, double* outputs);
int bes_mlp_apply_grad(bes_mlp* mlp, const float* grad, double lr, double weight_decay);
int bes_mlp_normalisation(const bes_mlp* mlp, double* out);

/* Counters of the context: out[0] kernels launched (graph kernel nodes counted per graph
 * launch), out[1] explicit iterations, out[2] implicit steps, out[3] linear iterations,
 * out[4] linear iterations whose Gram-Schmidt step needed the second pass.  out [5]. */
int bes_counters(const bes_ctx* ctx, int64_t* out);

/* FP64 fused multiply-add rate of the current device (FMA per second), measured with
 * independent FMA chains on every SM: the denominator of the explicit kernels' roofline. */
int bes_fp64_fma_rate(double* fma_per_s);

/* Library build identification (e.g. "sm_103a"). */
const char* bes_build_info(void);

/* ---- Output files and the solve loop ------------------------------------------------
 * The reference's writers, text for text (SolutionSnapshot::writePrimitiveToVtk / ToCsv /
 * writeSlipWallToCsv, src/SolutionSnapshot.cpp:145-309): default std::ostream formatting
 * (6 significant digits) of the "dimensional" primitives rho, Mach vector, gamma*p, gamma*R*T
 * (GasPerfect_<T>::convertDimensional, src/GasPerfect.tpp:294-326). */
#define BES_OUTPUT_VTK 0            /* solution as legacy ASCII VTK unstructured grid */
#define BES_OUTPUT_CSV 1            /* solution as CSV: centroid, 6 primitives per cell */
#define BES_OUTPUT_SLIP_WALL_CSV 2  /* slip-wall faces: centre, dimensional normal, owner's
                                       6 primitives (zeroth-order surface values) */

/* The .besi output keys (src/Config.cpp:155-187, 269-272). */
typedef struct {
  char folder[1024];      /* OUTPUT_FOLDER (default ".") */
  int32_t format;         /* OUTPUT_FORMAT: BES_OUTPUT_VTK (default) or BES_OUTPUT_CSV */
  int32_t slip_wall;      /* OUTPUT_SLIP_WALL: 1 YES, 0 NO (default) */
  int64_t save_interval;  /* SAVE_INTERVAL: files after step k when k % SAVE_INTERVAL == 0
                             and after the last step; 0 (default): after the last step only
                             (the reference leaves it unset and divides by it) */
  int32_t verbose;        /* 1: print the reference's console table to stdout */
  int32_t reserved;
} bes_output;

void bes_output_default(bes_output* out);

/* The output keys of a .besi file (other keys are left to bes_options_from_besi).  Same
 * token rules as Config::readConfigFile_; a bad OUTPUT_FORMAT / OUTPUT_SLIP_WALL value ->
 * BES_ERR_CONFIG. */
int bes_output_from_besi(const char* besi_path, bes_output* out, char* err, size_t err_cap);

/* Write the context's current state to `path` (kind BES_OUTPUT_*).  The VTK title line is
 * `path`, as in the reference, which passes its own file name. */
int bes_write(bes_ctx* ctx, const char* path, int32_t kind);

/* Host-only (no GPU) form of bes_write for a state U [n_cells][5] in reference numbering;
 * builds the reference-semantics mesh from `mesh` (gas constants and the MUSCL option from
 * `opt`). */
int bes_write_host(const bes_mesh_arrays* mesh, const bes_options* opt, const double* U,
                   const char* path, int32_t kind, char* err, size_t err_cap);

/* Solver::solve (src/SolverExplicit.cpp:395-438, src/SolverImplicit.cpp:552-600):
 * NUMBER_OF_TIME_STEP steps of the context's solver from its current state.  residual.csv in
 * out->folder is truncated, then every step appends "<step>," and the line the reference's
 * timeStep_ logs (explicit: max |R| per variable of the last stage; implicit: max |RHS| per
 * variable, linear iterations, linear error; "%e," formatting); solution_<step>.vtk|csv and
 * (OUTPUT_SLIP_WALL) slip_wall_<step>.csv are written after the steps save_interval selects. */
int bes_solve(bes_ctx* ctx, const bes_output* out);

/* Checkpoint and resume (no counterpart in the reference, which has no restart reader and
 * writes output snapshots only, src/SolverExplicit.cpp:427-433).  save writes the FP64 state of
 * every condition, each condition's freestream, active flag, CFL controller and step counters,
 * and the explicit step counter to a binary file; load restores them into a context created
 * with the same mesh, solver type and condition count, which then continues bit for bit as
 * the saved one would have.  BES_ERR_INVALID (with a message) for an unreadable or
 * mismatched file. */
int bes_checkpoint_save(bes_ctx* ctx, const char* path);
int bes_checkpoint_load(bes_ctx* ctx, const char* path);

/* Sizes of the ABI structs as compiled: out[0] = sizeof(bes_options),
 * out[1] = sizeof(bes_mesh_arrays), out[2] = sizeof(bes_output).  out [3].  Lets a binding
 * check its struct mirrors. */
void bes_abi_sizes(int64_t* out);

/* Host-only (no GPU): the mesh part of bes_create — face discovery, geometry and renumbering —
 * returned in reference numbering (Mesh::initialize, src/Mesh.cpp:66-93).  Call with NULL
 * arrays to obtain n_cells / n_faces first.  volume [n_cells], centroid [n_cells][3],
 * face_S [n_faces][3] (dimensional normal), face_area [n_faces], face_owner / face_neigh
 * [n_faces] (-1 on boundary), face_kind [n_faces] (0 internal, 1 slip wall, 2 freestream),
 * muscl_slot [n_cells][4] (local face whose vector the MUSCL reconstruction uses),
 * cell_new2ref [n_cells] / face_new2ref [n_faces] (the library's internal orders).  Any array
 * may be NULL. */
int bes_host_geometry(const bes_mesh_arrays* mesh, int32_t muscl_face_vector, int64_t* n_cells,
                      int64_t* n_faces, double* volume, double* centroid, double* face_S,
                      double* face_area, int64_t* face_owner, int64_t* face_neigh,
                      int64_t* face_kind, int64_t* muscl_slot, int64_t* cell_new2ref,
                      int64_t* face_new2ref, char* err, size_t err_cap);

/* Host-only (no GPU): 64-bit digests (FNV-1a) of every device-layout array the mesh build
 * produces (numbering, cell and face arrays, ELL slots, colouring and the block-ILU(0)
 * schedule; rcm_ilu_order 1: the level-scheduled RCM order), so that builds on different
 * thread counts or hosts can be compared array for array.  *n receives the count (30);
 * digests [cap] may be NULL. */
int bes_host_layout_digest(const bes_mesh_arrays* mesh, int32_t muscl_face_vector,
                           int32_t rcm_ilu_order, uint64_t* digests, int32_t cap, int32_t* n,
                           char* err, size_t err_cap);

#ifdef __cplusplus
}
#endif

#endif /* BES_GB300_H */
