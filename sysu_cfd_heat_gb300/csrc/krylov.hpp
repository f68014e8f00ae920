// Sparse matrices and Krylov solvers on the GPU.
//
// Storage is SELL-32: rows are grouped in slices of 32 (one warp), each slice
// padded to its longest row and stored column-major, so that the 32 lanes of a
// warp read consecutive values and column indices.  Entry k = 0 of every row
// is its diagonal; the remaining entries follow in the order the assembly
// kernels write them.  Padding entries point at the row itself with value 0.
//
// The solvers replace LASPack's CGIter / BiCGSTABIter as called through
// SolveLinearEqu (tools.cpp:56-64): same stopping test ||b-Ax||/||b|| < eps on
// the unpreconditioned residual recurrence, same iteration cap, Jacobi
// preconditioner y = omega D^-1 c.  Each solve is one cooperative launch of a
// persistent kernel; iteration counts and residuals stay on the device.
#pragma once

#include <vector>

#include "device.hpp"

namespace sysu {

struct SellPattern {
    int n = 0, nslices = 0;
    long nnz = 0;      // stored entries including padding
    long nnz_true = 0; // entries excluding padding
    std::vector<int> sl_ptr, sl_w, col;
    // row_len[i] = number of true entries of row i
    std::vector<int> row_len;
    // position of (row, k) in the value array
    long pos(int row, int k) const { return (long)sl_ptr[row >> 5] + (long)k * 32 + (row & 31); }
};

// Build a SELL-32 pattern from per-row column lists (diagonal first).
SellPattern make_sell(int n, const std::vector<int> &row_ptr, const std::vector<int> &cols);

// Level schedule of a pattern in natural row order, for the triangular sweeps of
// SSOR and ILU(0): forward level of row i = 1 + the largest forward level among
// its columns j < i; backward level = 1 + the largest among its columns j > i.
// Rows of one level do not depend on each other.  Rows are stored grouped by
// level (ascending row number inside a level).
struct LevelSchedule {
    int nf = 0, nb = 0;  // number of forward / backward levels
    DevBuf<int> fptr, frows, bptr, brows;
    // per level-ordered row: {row, SELL position of its entry 0, slice width, 0},
    // so a sweep reads everything it needs to start a row in one 16-byte load
    DevBuf<int4> finfo, binfo;
};

struct SellDev {
    int n = 0, nslices = 0;
    int wmax = 0;      // widest slice (entries per row incl. padding)
    long nnz = 0, nnz_true = 0;
    DevBuf<int> sl_ptr, sl_w, col;
    LevelSchedule lev;
    void upload(const SellPattern &p, cudaStream_t s);
};

// View passed to kernels.
struct SellView {
    int n, nslices;
    const int *sl_ptr, *sl_w, *col;
    const double *val;
};

struct SolveInfo {
    int status[3];
    int iters[3];
    double res[3];
    int err;
    int refinements;  // mixed precision: FP64 defect-correction sweeps
};

// Scratch of the persistent solvers, sized for n rows and up to 3 RHS.
struct KrylovWork {
    int n = 0, nrhs = 0, max_blocks = 0;
    DevBuf<double> r, rt, p, v, s, t, dinv, partials;
    DevBuf<double> sval;  // BiCGSTAB: matrix values scaled by the Jacobi diagonal inverse of their column
    DevBuf<float> r32, z32, p32, q32, e32, dinv32;  // mixed-precision inner solve
    DevBuf<float> rt32, v32, s32, t32, sval32;      // mixed BiCGSTAB (with r32, p32, e32)
    DevBuf<double> gV, gZ, gW, ilu;                  // GMRES basis, preconditioned basis, ILU(0) factors
    DevBuf<long long> gpart;                         // exact multi-value partial sums
    DevBuf<GridBarrier> barrier;
    unsigned long long *phase_ts = nullptr;  // optional: 4 timestamps per CG iteration, first 64
    // > 0: the persistent solves of this work use at most this many SMs' worth of
    // blocks (cases that share the GPU; the batch autotuner sets it)
    int sm_cap = 0;
    void ensure(int n, int nrhs, int max_blocks, cudaStream_t st);
    void ensure32(int n, cudaStream_t st);
};

struct KrylovOpts {
    int maxit = 500;
    double eps = 1e-8;
    double omega = 1.0;       // Jacobi weight (the omega LASPack's precond gets)
    bool jacobi = true;       // false: no preconditioner
    double inner_tol = 0.1;   // mixed precision: FP32 residual drop that triggers a reliable update
};

// Preconditioners of the general solvers (LASPack's JacobiPrecond, SSORPrecond,
// ILUPrecond; none = identity).  PK_AMG (the symmetric p' systems only):
// flexible CG with FP32 recurrences and FP64 reliable updates, preconditioned
// by the aggregation-multigrid V-cycle of amg.hpp.
enum PrecondKind { PK_NONE = 0, PK_JACOBI = 1, PK_SSOR = 2, PK_ILU0 = 3, PK_AMG = 4 };
constexpr int GMRES_MAX_RESTART = 30;

// Restarted GMRES(m), right preconditioned (the oracle's LASPack restatement:
// Saad Alg. 9.5 with Givens rotations), classical Gram-Schmidt applied twice with
// exact deterministic grid sums; stopping test ||b - A x|| / ||b|| < eps, checked
// on the true residual at the end of a cycle.  restart in 1..GMRES_MAX_RESTART.
void gmres_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
                 const KrylovOpts &o, int precond, int restart, KrylovWork &w, SolveInfo *info_dev,
                 cudaStream_t st);

// Preconditioned CG with any PrecondKind (Templates Fig. 2.5).
void pcg_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
               const KrylovOpts &o, int precond, KrylovWork &w, SolveInfo *info_dev, cudaStream_t st);

// y = M^-1 c once (the LASPack preconditioner entry points).
void precond_solve(const SellDev &A, const double *val, int precond, double omega, const double *c, double *y,
                   KrylovWork &w, SolveInfo *info_dev, cudaStream_t st);

// Copy FP64 SELL values to FP32 (same pattern).
void sell_to_fp32(const SellDev &A, const double *val, float *val32, cudaStream_t st);

// Mixed precision CG: FP32 Jacobi-CG recurrences with reliable updates -- each
// time the FP32 residual has fallen by inner_tol, the FP32 correction is added
// to the FP64 x and the FP64 residual b - A x replaces the FP32 one, keeping
// the search direction (defect correction without restarting).  Dot products
// are summed in FP64 across threads.  Stops on the FP64 residual
// ||b - A x|| / ||b|| < eps; iters = FP32 iterations, refinements = updates.
void cg_solve_mixed(const SellDev &A, const double *val, const float *val32, const double *b, double *x,
                    bool x0_zero, const KrylovOpts &o, KrylovWork &w, SolveInfo *info_dev, cudaStream_t st);


// Jacobi-preconditioned CG; x holds x0 on entry (or is zeroed first if x0_zero).
void cg_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
              const KrylovOpts &o, KrylovWork &w, SolveInfo *info_dev, cudaStream_t st);

// The scratch bicgstab_solve needs for nrhs right-hand sides of one matrix,
// allocated ahead (a solve captured into a graph must not allocate).
void bicgstab_prepare(const SellDev &A, int nrhs, KrylovWork &w, cudaStream_t st);

// BiCGSTAB on nrhs (1..3) right-hand sides sharing one matrix; b[c], x[c].
void bicgstab_solve(const SellDev &A, const double *val, int nrhs, const double *const *b, double *const *x,
                    const KrylovOpts &o, KrylovWork &w, SolveInfo *info_dev, cudaStream_t st);

// BiCGSTAB for one system with FP32 inner iterations (column-scaled FP32 matrix,
// Jacobi) in FP64 defect correction: x += M^-1 e and the FP64 residual b - A x
// once the FP32 residual fell by o.inner_tol; stops on ||b - A x|| / ||b|| < eps.
// x holds x0 on entry.
void bicgstab_solve_mixed(const SellDev &A, const double *val, const double *b, double *x, const KrylovOpts &o,
                          KrylovWork &w, SolveInfo *info_dev, cudaStream_t st);

// The momentum form of the mixed BiCGSTAB: u, v, w of one matrix (b[c], x[c]
// with x0 in) by one sequence of flat kernels with FP32 recurrences on vectors
// interleaved per row, x accumulated in FP64 every iteration, and the FP64
// residual b - A x replacing the FP32 one once it fell by o.inner_tol; stops
// each component on ||b - A x|| / ||b|| < eps.  A component whose replacements
// stop lowering that residual is finished by the FP64 batched BiCGSTAB from its
// x.  Per-component status, iterations (FP32) and residual in info; refinements
// = replacements summed over the components.  The solve never waits for the
// host: its iterations are a WHILE node of a CUDA graph (graph_loop.hpp), so on
// a stream being captured it joins the caller's graph, and otherwise it runs as
// its own graph (captured once, again when its arguments change).
class Bicg3Mixed {
  public:
    Bicg3Mixed();
    ~Bicg3Mixed();
    Bicg3Mixed(const Bicg3Mixed &) = delete;
    Bicg3Mixed &operator=(const Bicg3Mixed &) = delete;
    void solve(const SellDev &A, const double *val, const double *const *b, double *const *x, const KrylovOpts &o,
               KrylovWork &w, SolveInfo *info_dev, cudaStream_t st);
    // false: the host drives the iterations (a captured chunk of them, the state
    // read after each) -- for per-kernel profiling; profilers skip the kernels of
    // graphs with conditional nodes.  A capturing stream always gets the device loop.
    bool device_loop = true;

  private:
    struct Impl;
    Impl *d_;
};

// BiCGSTAB on three systems with one sparsity pattern and their own values
// vals[c] (and Jacobi diagonals), in one launch: the column indices are read
// once per product for the three (k, eps and T of one outer iteration).
void bicgstab_solve_multi(const SellDev &A, const double *const *vals, const double *const *b, double *const *x,
                          const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st);

// y = A x (standalone, for tests and the SpMV sweep).
void spmv(const SellDev &A, const double *val, const double *x, double *y, cudaStream_t st);

// y = A x with the matrix streamed once (evict-first loads), FP64 and FP32 values:
// the standalone SpMV of the sweep.
void spmv_stream(const SellDev &A, const double *val, const double *x, double *y, cudaStream_t st);
void spmv_stream32(const SellDev &A, const float *val, const float *x, float *y, cudaStream_t st);
// SpMV kernel form of spmv_stream / spmv_stream32: 0 one row per thread over a
// full grid; 10 b + s: b blocks of 256 per SM, s in {1, 2, 4} slices per warp step.
void set_spmv_variant(int v);
int spmv_variant();
constexpr int SPMV_RING = 100;   // spmv_variant value that selects spmv_ring in the sweep
constexpr int SPMV_ASYNC = 200;  // per-warp cp.async pipeline (spmv_stream / spmv_stream32)
constexpr int SPMV_STAGE = 300;  // x staged in shared memory per block of rows (spmv_stream / spmv_stream32)
// y = A x by a persistent kernel that streams the matrix through a shared-memory
// ring with bulk copies (one CTA per SM; cg.cu).  *err (device) is set if a
// bounded wait in the ring gave up.  val and the column indices 16-byte aligned.
void spmv_ring(const SellDev &A, const double *val, const double *x, double *y, int *err, cudaStream_t st);
void spmv_ring32(const SellDev &A, const float *val, const float *x, float *y, int *err, cudaStream_t st);
// L2 flush by reading `bytes` (> L2) of buf: clean lines, no write-back later.
void l2_flush_read(const void *buf, size_t bytes, unsigned *sink, cudaStream_t st);
// x of the sweep (FP64 and its FP32 copy).
void fill_sweep_x(long n, double *x64, float *x32, cudaStream_t st);

// y = omega D^-1 c (the Jacobi preconditioner applied once).
void jacobi_apply(const SellDev &A, const double *val, double omega, const double *c, double *y, cudaStream_t st);

}  // namespace sysu
