/*
 * sysu_cfd.h -- C ABI of the GB300-native SIMPLE solver (libsysucfd.so).
 *
 * This is the solver-level drop-in boundary: the entry points below replace
 * the reference's NavierStokesSolver / HeatConductionSolver driver sequence
 * (reference src/main.cpp:8-33) and its SIMPLE outer loop
 * (src/navier.cpp:13-97).  Inputs are the reference's own formats: a
 * param.in keyword file (src/readparamfile.cpp:10-260) naming a Gmsh MSH 2.x
 * ASCII mesh (src/Preprocessor.cpp:13-146).  All fields live on one GPU;
 * host copies are made only on request.
 *
 * Conventions: plain pointers and sizes, int status codes (SYSU_OK = 0), the
 * message of the last failure through sysu_last_error().  One solver per host
 * thread; the library keeps no global state besides the error message
 * (thread-local).  Nothing here exits the process: where the reference calls
 * exit()/fatalRuntimeError, these functions return SYSU_ERR_SOLVE or
 * SYSU_ERR_INPUT with the reference's message.
 */
#ifndef SYSU_CFD_H
#define SYSU_CFD_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SYSU_OK 0
#define SYSU_ERR_INPUT 1  /* bad param file / mesh / argument */
#define SYSU_ERR_CUDA 2   /* CUDA runtime error (no device, launch failure) */
#define SYSU_ERR_SOLVE 3  /* a convergence check of the reference failed */

typedef struct sysu_case sysu_case;
typedef struct sysu_solver sysu_solver;

const char *sysu_last_error(void);
int sysu_version(void);

/* ---- host-only case access (needs no GPU) --------------------------------
 * Parses param.in, reads the mesh, builds faces in the reference's order
 * (Preprocessor.cpp:181-299), splits fluid and solid for conjugate heat
 * transfer (Preprocessor.cpp:308-515) and computes the geometry of
 * CycasSolver::CellFaceInfo (BasicSolver.cpp:317-512). */
int sysu_case_load(const char *param_path, sysu_case **out);
void sysu_case_free(sysu_case *c);
/* out[0..11] = fluid Ncel, Nfac, Nbnd, Nvrt, NCoupledBnd, solid Ncel, Nfac,
 * Nbnd, Nvrt, NCoupledBnd, has_solid, coupled region id */
int sysu_case_info(const sysu_case *c, long *out, int n);
/* Copy a geometry/topology array by name ("cell_vol", "cell_x", "face_n",
 * "face_lambda", "bnd_distance", ...; prefix "solid_" for the solid).
 * Returns the array's size in bytes (or -1 for an unknown name); copies
 * min(size, nbytes) bytes when out is non-null. */
long sysu_case_array(const sysu_case *c, const char *name, void *out, long nbytes);
/* The Tecplot writer on host arrays (no GPU): fields by name "P" "U" "V" "W" "R"
 * "T" "VisLam" "VisTur" (required), "TE" "ED" (turbulence ke), "solid_T" (CHT),
 * in reference cell order. */
int sysu_case_write_tecplot(const sysu_case *c, const char *path, int nfields, const char *const *names,
                            const double *const *arrays);

/* ---- GPU solver ------------------------------------------------------------
 * create: main.cpp:14-28 (read, build, CellFaceInfo, CheckAndAllocate,
 * InitFlowField) with every field uploaded to the current CUDA device. */
int sysu_solver_create(const char *param_path, sysu_solver **out);
/* Wall-clock seconds of the last case preprocessing on this thread (solver or
 * case creation): out[0] MSH read, [1] face construction, [2] fluid/solid split,
 * [3] geometry (CellFaceInfo); out[4] = host threads used (SYSU_THREADS or the
 * hardware count; the results do not depend on it). */
int sysu_setup_phases(double *out);
/* Page-locked host memory for field transfers (sysu_solver_get_field /
 * set_field copy it by DMA; pageable memory works too, through the driver's
 * staging). NULL on failure. */
void *sysu_host_alloc(size_t bytes);
void sysu_host_free(void *p);
void sysu_solver_destroy(sysu_solver *s);
/* out[0..5] = Ncel, Nfac, Nbnd, solid Ncel, matrix stored entries, matrix true entries */
int sysu_solver_info(sysu_solver *s, long *out, int n);
/* Options (defaults = the reference's call sites):
 *   "<eq>.eps" "<eq>.maxit" "<eq>.omega" "<eq>.kind" (0 CG, 1 BiCGSTAB, 2 GMRES)
 *     "<eq>.precond" (0 none, 1 Jacobi, 2 SSOR, 3 ILU(0); SSOR/ILU with CG and
 *     GMRES) "<eq>.restart" (GMRES, 1..30) for eq in mom, p, ke, t, ts (solid T);
 *   "reference_solvers" (1: the reference's own mode, GMRES(10) + SSOR for
 *     momentum, k, eps, T and CG + SSOR for p' and solid T; 0: back to the
 *     default mode, BiCGSTAB + Jacobi and CG + Jacobi, which reach the same
 *     solutions to the tolerance and are faster on the GPU);
 *   "<eq>.mixed" (FP32 recurrences, stopping on the FP64 residual: p and ts
 *     by CG with FP64 reliable updates; mom, ke, t by BiCGSTAB -- momentum with
 *     mom_batched as one solve of u, v, w on interleaved FP32 vectors with FP64
 *     residual replacement, otherwise one system after another with FP32 inner
 *     iterations in FP64 defect correction; not with GMRES) and
 *     "<eq>.inner_tol" (0 < inner_tol < 1: the FP32 residual drop between FP64
 *     residuals; 0.1, 1e-4 for mom);
 *   "p.learned" (1: the p' CG with the learned preconditioner -- the first
 *     "p.learn_iters" solves run the plain method and train the network on
 *     their residual/correction pairs, "p.learn_steps" Adam steps each at rate
 *     "p.learn_lr" with loss "p.learn_kind" (0 energy norm, 1 residual norm);
 *     later solves run flexible CG with the network, see sysu_gnn_fcg; the
 *     network survives sysu_solver_reset; read-only "p.learned_solves");
 *   "scalars_batched" (1: k, eps and T assembled together and solved by one
 *     batched BiCGSTAB launch; eps's source and T's conductivity then lag by
 *     one outer iteration, the steady solution is the same; needs ke + energy);
 *   "sm_cap" (SMs' worth of blocks the persistent Krylov solves may use, 0 = all;
 *     set per case by the batch autotuner);
 *   "rtc" sets every eq's eps; "mom_batched" (1: u,v,w as one 3-RHS solve);
 *   "graph_loops" (1, default: the mixed momentum and the multigrid p' solves
 *     loop on the device as CUDA graph WHILE nodes, which lets them run inside a
 *     captured graph; 0: the host drives those loops -- for per-kernel profiling,
 *     since profilers skip the kernels of graphs with conditional nodes);
 *   "solid_source" (W/m^3, an extension); "fatal_checks"; "timing". */
int sysu_solver_set_option(sysu_solver *s, const char *key, double value);
int sysu_solver_get_option(sysu_solver *s, const char *key, double *value);
/* Run up to n bodies of the steady NSSolve loop (navier.cpp:33-68): velocity,
 * pressure, k-epsilon, energy and solid conduction as configured.  Stops
 * early when max(Residual) < ResidualSteady.  *done = iterations run. */
int sysu_solver_iterate(sysu_solver *s, int n, int *done);
/* NSSolve itself.  Steady: MaxOuterStep-1 iterations with the steady break.
 * Transient ("transient, dt, total, Euler|Dual, MaxOuterStep"): time steps of
 * outer iterations with the reference's break rule (navier.cpp:29-88);
 * *done = outer iterations run in all steps.  With option
 * "output" on it also writes what the reference writes next to param.in:
 * tot.dat (header, then one VolumnAverage line), tec/res%04lu.dat every
 * `output, N` iterations (navier.cpp:59-61,104-110) and once at the end. */
int sysu_solver_nssolve(sysu_solver *s, int *done);
/* NavierStokesSolver::Output (navier.cpp:264-337, plus the solid zone of
 * HeatConductionSolver.cpp:330-361): <dir>/tec/res%04lu.dat, numbered per
 * solver from 0, text identical to the reference's.  dir NULL = the directory
 * of param.in. */
int sysu_solver_output(sysu_solver *s, const char *dir);
/* NavierStokesSolver::VolumnAverage (navier.cpp:243-261): one line appended to
 * <dir>/tot.dat (created with the reference's header when missing). */
int sysu_solver_volume_average(sysu_solver *s, const char *dir, double t, int out_iter);
/* The individual methods, enqueued on the solver's stream (navier.h:103-116):
 * CalculateVelocity, CalculatePressure, UpdateTurKEpsilon, UpdateEnergy,
 * HeatConductionSolver::solve.  sysu_solver_check() then reads the residuals
 * and applies the reference's convergence checks. */
int sysu_solver_calculate_velocity(sysu_solver *s);
int sysu_solver_calculate_pressure(sysu_solver *s);
int sysu_solver_update_turkeps(sysu_solver *s);
int sysu_solver_update_energy(sysu_solver *s);
int sysu_solver_heat_conduction(sysu_solver *s);
/* CycasSolver::SaveTransientOldData of the fluid and the solid module
 * (navier.cpp:190-240, HeatConductionSolver.cpp:306-327): the current fields
 * become the previous time level (a transient case; no-op when steady). */
int sysu_solver_save_transient_old_data(sysu_solver *s);
int sysu_solver_check(sysu_solver *s);
/* Back to the state right after creation (InitFlowField); keeps the mesh,
 * matrices and options. */
int sysu_solver_reset(sysu_solver *s);
/* CUDA events on the solver's stream: start, then stop returns the elapsed
 * device time in ms (stop synchronises). */
int sysu_solver_timer_start(sysu_solver *s);
int sysu_solver_timer_stop(sysu_solver *s, double *ms);
/* Number of kernels the library has launched so far (all solvers). */
long sysu_kernel_launches(void);
/* With option "profile_phases" on: %globaltimer stamps (ns) taken by block 0
 * of the last CG solve at the start of each iteration, after the direction
 * update, after the product + reduction and after the update + reduction --
 * 4 per iteration for the first 64 iterations (n <= 256). */
int sysu_solver_cg_phases(sysu_solver *s, unsigned long long *out, int n);
/* Standalone SpMV sweep on an assembled matrix ("mom", "p", "scalar", "solid"):
 * *ms = mean device time of one y = A x (streaming SELL-32 kernel) over `reps`
 * products on a fixed x, FP64 values or (fp32 != 0) their FP32 copy, with L2
 * flushed before every product. */
int sysu_solver_spmv_timing(sysu_solver *s, const char *which, int fp32, int reps, double *ms);
/* The same product timed in steady state: 2 * max(reps, 2) products back to back,
 * alternating between the matrix (values, column indices, slice table) with its x
 * and y and a full copy of all of them -- more than the L2 holds for the 2M-row
 * systems, so each product reads its operands from HBM as one inside an iterative
 * solve does, without the launch ramp and tail of a single timed product.
 * *ms = mean per product. */
int sysu_solver_spmv_timing_steady(sysu_solver *s, const char *which, int fp32, int reps, double *ms);
/* Residual[0..9] of the last iteration (navier.h:65). */
int sysu_solver_residuals(sysu_solver *s, double *out10);
/* Per solve slot (mom u/v/w, p', k, eps, T, solid T): iterations, residual,
 * status (0 converged, 1 max iterations, 2 breakdown, 3 barrier timeout,
 * 4 non-finite).  Arrays of 6*3 entries, slot-major. */
int sysu_solver_solve_stats(sysu_solver *s, int *iters, double *res, int *status);
/* CUDA-event times of the last p' and momentum solves (option "timing"). */
int sysu_solver_timing(sysu_solver *s, double *p_ms, double *mom_ms);
/* Fields by the reference's member names: cell fields "U" "V" "W" "P" "R"
 * "T" "TE" "ED" "VisLam" "VisTur" "Apr"; gradients "dUdX" "dVdX" "dWdX"
 * "dPdX" "dPhidX" (3 per cell, cell-major); "RUFace" (reference face order);
 * boundary arrays "BU" "BV" "BW" "BRo" "BPre" "BTem" "BTE" "BED" "Bq";
 * "dp" (last p'), "bp" (its right-hand side), "b3"/"x3" (momentum right-hand
 * sides / solutions, 3*Ncel component-major); solid: "solid_T" "solid_dPhidX" "solid_BTem" "solid_Bq".
 * n must equal the field's size (sysu_solver_field_size). */
long sysu_solver_field_size(sysu_solver *s, const char *name);
int sysu_solver_get_field(sysu_solver *s, const char *name, double *out, long n);
int sysu_solver_set_field(sysu_solver *s, const char *name, const double *in, long n);
int sysu_solver_sync(sysu_solver *s);
/* The p' multigrid form (option p.precond 4; no counterpart in the reference,
 * whose p' solve is CG + SSOR, navier_pressure.cpp:29).  sysu_solver_p_cycle:
 * z = M r, one application of the cycle as the last p' solve left it (its
 * matrix values, and its network on its level when use_net).
 * sysu_solver_p_network: the level of the p' network (0 the finest, >= 1 a
 * coarse level of the cycle) and, when params is not NULL, its np =
 * sysu_gnn_num_params() parameters; sysu_solver_p_set_network replaces them. */
int sysu_solver_p_cycle(sysu_solver *s, const double *r, double *z, int use_net);
int sysu_solver_p_network(sysu_solver *s, int *level, float *params, int np);
int sysu_solver_p_set_network(sysu_solver *s, const float *params, int np);
/* Assembled matrix "mom", "p", "scalar" (last k/eps/T) or "solid" as CSR,
 * diagonal first in each row.  With rowptr == NULL returns the entry count;
 * otherwise fills rowptr[n+1], col[], val[] and returns the count (-1: error). */
long sysu_solver_matrix(sysu_solver *s, const char *which, int *rowptr, int *col, double *val);

/* ---- standalone sparse solves on the GPU ------------------------------------
 * The Krylov kernels of the SIMPLE path applied to a host CSR matrix (0-based,
 * any column order).  method: 0 CG, 1 BiCGSTAB, 2 CG with FP32 recurrences and
 * FP64 reliable updates (Jacobi only; iters = FP32 iterations), 3 GMRES(10)
 * right preconditioned, 4 BiCGSTAB with FP32 inner iterations in FP64 defect
 * correction (none or Jacobi; iters = FP32 iterations), 5 flexible CG with FP32
 * recurrences and FP64 reliable updates preconditioned by the aggregation-
 * multigrid V-cycle (symmetric matrices; precond 4, omega = the smoother's
 * Jacobi weight, 0.8 suits the p' systems; iters = FP32 iterations);
 * precond: 0 none, 1 Jacobi (y = omega D^-1 c), 2 SSOR(omega),
 * 3 ILU(0) (level-scheduled sweeps; not with BiCGSTAB), 4 multigrid (method 5 only).  Stopping test ||b - A x||_2 / ||b||_2 < eps, as the
 * reference's SolveLinearEqu (tools.cpp:56-64) expects.  x: x0 in, solution out.
 * status: 0 converged, 1 max iterations, 2 breakdown, 3 barrier timeout,
 * 4 non-finite (a mixed solve whose FP32 refinement stalls is finished by the
 * FP64 method from its current x; the status is then the FP64 one). */
int sysu_csr_solve(int method, int precond, int n, const int *rowptr, const int *col, const double *val,
                   const double *b, double *x, int maxit, double eps, double omega, int *iters, double *res,
                   int *status);
int sysu_csr_spmv(int n, const int *rowptr, const int *col, const double *val, const double *x, double *y);
/* Kernel form of the standalone SpMV (sysu_csr_spmv and the sweep of
 * sysu_solver_spmv_timing), process-wide: 0 one row per thread over a full
 * grid (default), 100 persistent ring (matrix streamed through shared memory
 * by bulk copies, one CTA per SM), 200 per-warp cp.async pipeline staging the
 * next slices in shared memory, 300 x staged in shared memory per block of 256
 * rows (the rows' window plus a 96-row halo; other columns read from global
 * memory), 10 b + s the persistent grid with s slices
 * per warp step and b blocks per SM.  All forms give bit-identical y. */
int sysu_set_spmv_variant(int variant);
/* Mean device ms of one y = A x of a host CSR matrix by the current kernel form
 * (FP64 values, or their FP32 copy when fp32), L2 flushed before each of `reps`
 * timed products (the procedure of the solver's SpMV sweep). */
int sysu_csr_spmv_timing(int n, const int *rowptr, const int *col, const double *val, int fp32, int reps,
                         double *ms);
/* Three systems sharing one sparsity pattern (rowptr, col), values vals[c],
 * right-hand sides b[c], x[c] (x0 in, solution out), solved by one batched
 * BiCGSTAB + Jacobi launch (the k, eps, T form of option "scalars_batched"). */
int sysu_csr_bicgstab_batched3(int n, const int *rowptr, const int *col, const double *const *vals,
                               const double *const *b, double *const *x, int maxit, double eps, int *iters,
                               double *res, int *status);
/* Three right-hand sides b[c] of one matrix (the momentum form: u, v, w of
 * navier_velocity.cpp:26, solved there one after another by BiCGSTABIter),
 * x[c] x0 in and solution out, BiCGSTAB + Jacobi (omega D^-1).  mixed 0: the
 * FP64 batched solve of the SIMPLE path; mixed 1: FP32 recurrences on the
 * three vectors interleaved per row, x accumulated in FP64, the FP64 residual
 * b - A x replacing the FP32 one once that fell by inner_tol (0 < inner_tol < 1),
 * the stopping test ||b - A x|| / ||b|| < eps on it (a component whose
 * replacements stop lowering it is finished by the FP64 solve).  iters, res,
 * status: 3 each; refinements: replacements summed over the components. */
int sysu_csr_bicgstab3(int n, const int *rowptr, const int *col, const double *val, const double *const *b,
                       double *const *x, int mixed, int maxit, double eps, double omega, double inner_tol,
                       int *iters, double *res, int *status, int *refinements);
/* Self-test of the device-side solve loops (CUDA graph WHILE nodes, whose
 * last kernel ends the loop when the solve's stop flag is set or after a bound of
 * bodies): *bodies = the number of bodies run when the flag is set after stop_at
 * bodies (never, for stop_at <= 0) and the bound is `bound`; min(stop_at, bound). */
int sysu_graph_loop_selftest(int bound, int stop_at, int *bodies);
const char *sysu_csr_last_error(void);

/* ---- aggregation-multigrid hierarchy (host only, no device work) -----------
 * No counterpart in the reference (its p' solve is CG + SSOR,
 * navier_pressure.cpp:29).  The hierarchy that p' option precond 4 and method 5
 * build, for a host CSR matrix: greedy aggregation at strength threshold theta,
 * Galerkin coarse levels until a level has at most dense_max rows.
 * sysu_mg_hierarchy: number of levels, rows and entries per level (up to
 * max_levels).  sysu_mg_level: aggregate of each row of `level` (agg, may be
 * NULL) and that level's matrix as CSR with the diagonal first (rowptr_out of
 * rows + 1, col_out / val_out of the level's entry count; may be NULL). */
int sysu_mg_hierarchy(int n, const int *rowptr, const int *col, const double *val, double theta, int dense_max,
                      int max_levels, int *nlevels, int *rows, long *nnz);
int sysu_mg_level(int n, const int *rowptr, const int *col, const double *val, double theta, int dense_max,
                  int level, int *agg, int *rowptr_out, int *col_out, double *val_out);
const char *sysu_mg_last_error(void);

/* ---- Jacobi-CG that allocates nothing ----------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * applications that own all device memory through their own pool and do not
 * let a library allocate behind their back, or loops that must not pay the
 * device-wide synchronisation of cudaMalloc/cudaFree.  The caller passes its
 * own DEVICE buffers: CSR d_rowptr[n+1], d_col[nnz], d_val[nnz] (0-based), d_b[n],
 * d_x[n] (x0 in, solution out); same algorithm and stopping test as
 * sysu_csr_solve with method CG and precond Jacobi.  Scratch is one static
 * device array of 8.4 MB, present on every GPU that loads the library:
 *   - n must be <= SYSU_NOALLOC_MAX_ROWS, larger systems are rejected
 *     (SYSU_ERR_INPUT, message in sysu_noalloc_last_error());
 *   - every call shares the array; calls that overlap on the GPU race on it;
 *   - every call looks the array's address up (cudaGetSymbolAddress, which
 *     allocates nothing) with the calling thread's device current;
 *   - every call waits for its stream to read iters / res / status back, so it
 *     cannot be captured into a CUDA graph: on a capturing stream it returns
 *     SYSU_ERR_INPUT and queues nothing;
 *   - the CSR is the caller's responsibility; rows whose pointer decreases,
 *     columns outside 0..n-1 and rows without a nonzero diagonal are detected
 *     on the device and returned as SYSU_ERR_INPUT (lowest such row in the
 *     message) without solving; rowptr[n] must not exceed the length of
 *     d_col / d_val, which the call cannot check.
 * stream: a cudaStream_t (NULL = default stream). */
#define SYSU_NOALLOC_MAX_ROWS 262144
int sysu_csr_cg_noalloc(int n, const int *d_rowptr, const int *d_col, const double *d_val, const double *d_b,
                        double *d_x, int maxit, double eps, double omega, void *stream, int *iters, double *res,
                        int *status);
const char *sysu_noalloc_last_error(void);

/* ---- batches of independent cases -----------------------------------------
 * Many cases (each its own param.in) advanced together: sysu_batch_capture
 * records one outer iteration of every case into one CUDA graph (each case on
 * its own branch, so the cases run concurrently; the host is not involved
 * inside a replay); sysu_batch_replay(n) replays it n times.  The autotuner
 * (sysu_batch_tune) times one outer iteration of each case alone for every
 * candidate SM cap (the SMs' worth of blocks its persistent Krylov solves may
 * use -- the rows per warp of those kernels), then raises caps one step at a
 * time where that lowers the model makespan max(slowest case, SM-time / SMs),
 * while the caps add up to at most the GPU's SM count; the graph then issues
 * the longest cases first; finally the model's caps scaled by 1/2, 1, 2, 4 and 8
 * are each captured and replayed, and the fastest is kept (*makespan = its
 * measured ms per batch iteration).  It resets the cases afterwards.  Cases are reached with sysu_batch_case (borrowed handles:
 * options, fields, solve statistics; do not destroy them).  Capture after every
 * option change.  sysu_batch_run_sequential times the cases one after another
 * with ordinary launches, for comparison. */
typedef struct sysu_batch sysu_batch;
int sysu_batch_create(int n, const char *const *params, sysu_batch **out);
void sysu_batch_free(sysu_batch *b);
int sysu_batch_size(sysu_batch *b);
sysu_solver *sysu_batch_case(sysu_batch *b, int k);
/* caps/ms_alone/ms_full: one value per case (may be NULL) */
int sysu_batch_tune(sysu_batch *b, const int *cand, int ncand, int *caps, double *ms_alone, double *ms_full,
                    double *makespan);
int sysu_batch_set_caps(sysu_batch *b, const int *caps);
int sysu_batch_capture(sysu_batch *b);
int sysu_batch_replay(sysu_batch *b, int n, double *ms);
/* the reference's convergence checks on every case's last iteration */
int sysu_batch_check(sysu_batch *b);
int sysu_batch_run_sequential(sysu_batch *b, int n, double *ms);

/* ---- learned preconditioner (message-passing network) -----------------------
 * No counterpart in the reference: a 4-layer, width-32 message-passing network
 * over the graph of a symmetric matrix (for the p' systems: the cell-face
 * graph), BF16 weights with FP32 accumulation on the tensor cores, used as the
 * preconditioner of flexible CG.  z = s (u + w_d . h4 + b_d) with u = D^-1 r / s
 * and s = rms(D^-1 r); with zero decoder weights it is the Jacobi
 * preconditioner.  Parameters: a flat FP32 vector of sysu_gnn_num_params()
 * values, layout [e(32) c(32)] [W_l (64 x 32, input-major) b_l (32)] x 4
 * [w_d(32) b_d].  The handle owns a stream and the matrix on the device.
 * Training pairs (r, e = A^-1 r) go into a ring of `capacity` pairs; each
 * training step is one Adam step (beta 0.9 / 0.999) on one pair, in the
 * order the pairs were added; loss_kind 0 = energy norm of the error,
 * 1 = residual norm.  All calls return 0 or an error code (message in
 * sysu_gnn_last_error()). */
typedef struct sysu_gnn sysu_gnn;
int sysu_gnn_num_params(void);
int sysu_gnn_create(int n, const int *rowptr, const int *col, const double *val, int capacity, sysu_gnn **out);
void sysu_gnn_free(sysu_gnn *g);
/* new matrix values with the pattern given to sysu_gnn_create (same rowptr, col) */
int sysu_gnn_set_values(sysu_gnn *g, const int *rowptr, const int *col, const double *val);
int sysu_gnn_init_params(sysu_gnn *g, unsigned long long seed);
int sysu_gnn_set_params(sysu_gnn *g, const float *p, int np);
int sysu_gnn_get_params(sysu_gnn *g, float *p, int np);
/* z = M(r), host vectors of n values. */
int sysu_gnn_apply(sysu_gnn *g, const double *r, double *z);
int sysu_gnn_add_pair(sysu_gnn *g, const double *r, const double *e);
/* loss and gradient (np values) of pair k, no update */
int sysu_gnn_loss_grad(sysu_gnn *g, int k, int loss_kind, double *loss, float *grad, int np);
/* `steps` Adam steps cycling over the stored pairs; losses[steps] (may be NULL) */
int sysu_gnn_train(sysu_gnn *g, int steps, double lr, int loss_kind, double *losses);
/* Flexible CG (FP32 recurrences, FP64 reliable updates every inner_tol drop of
 * the residual) with the network (use_gnn = 1) or Jacobi as preconditioner.
 * Jacobi takes over when the network stalls for stall_max iterations or a
 * direction loses positivity (fallback_at = iteration, else -1).  Stops on
 * ||b - A x||_2 / ||b||_2 < eps.  x: x0 in (ignored if x0_zero), solution out.
 * seconds: device time of the solve (CUDA events). */
int sysu_gnn_fcg(sysu_gnn *g, const double *b, double *x, int x0_zero, int maxit, double eps, double inner_tol,
                 int use_gnn, int stall_max, int *iters, double *res, int *status, int *fallback_at,
                 int *refinements, double *seconds);
/* Multigrid form (no counterpart in the reference): on = 1 builds the
 * aggregation-multigrid hierarchy of the handle's matrix (strength theta,
 * smoother weight omega, coarse-correction scale gamma) and attaches it: from
 * then on sysu_gnn_fcg is preconditioned by the V-cycle whose finest
 * post-smoothing step is the network (use_gnn = 1) or Jacobi (use_gnn = 0);
 * the network's decoder then weighs its Jacobi term by omega, so a network
 * with a zero decoder is exactly the Jacobi step, and
 * sysu_gnn_set_values refreshes its coarse levels, and pairs added with
 * sysu_gnn_add_pair become pairs of the post-smoother,
 * (r, e) -> (r - A z2(r), e - z2(r)) with z2 the cycle before post-smoothing.
 * levels / rows (up to max_levels; may be NULL) report the hierarchy.
 * on = 0 detaches it. */
int sysu_gnn_set_multigrid(sysu_gnn *g, int on, double theta, double omega, double gamma, int *levels, int *rows,
                           int max_levels);
/* z = M(r): one application of the attached cycle (host vectors of n values) */
int sysu_gnn_mg_apply(sysu_gnn *g, const double *r, double *z, int use_gnn);
/* hidden state h^layer (layer 1..4) of the network on r, FP32 [n][32] */
int sysu_gnn_hidden(sysu_gnn *g, const double *r, int layer, float *h);
/* device ms of one network application on r (mean of reps); fwd_per_sm > 0
 * sets the forward kernel's CTAs per SM (0: derived from its registers) */
int sysu_gnn_time_apply(sysu_gnn *g, const double *r, int reps, int fwd_per_sm, double *ms);
const char *sysu_gnn_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
