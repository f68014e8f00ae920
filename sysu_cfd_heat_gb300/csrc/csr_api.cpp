// Standalone sparse entry points of the C ABI: solve / multiply with a
// host-side CSR matrix on the GPU, and read back an assembled matrix of a
// solver in CSR form.  They share the persistent Krylov kernels of the SIMPLE
// path (krylov.cu).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sysu_cfd.h"
#include "csr_device.hpp"
#include "gnn.hpp"
#include "graph_loop.hpp"
#include "handles.hpp"


namespace {
thread_local std::string g_csr_err;

// A non-blocking stream that is destroyed on every way out of the call,
// exceptions included.
struct OwnedStream {
    cudaStream_t st = nullptr;
    OwnedStream() { SYSU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)); }
    ~OwnedStream() {
        if (st) cudaStreamDestroy(st);
    }
    OwnedStream(const OwnedStream &) = delete;
    OwnedStream &operator=(const OwnedStream &) = delete;
};

// Argument errors (SYSU_ERR_INPUT) as opposed to CUDA/runtime errors.
struct ArgError {
    std::string msg;
};

void check_method(int method, int precond) {
    if (method < 0 || method > 5)
        throw ArgError{"method: 0 CG, 1 BiCGSTAB, 2 CG-mixed, 3 GMRES, 4 BiCGSTAB-mixed, 5 CG-multigrid"};
    if (precond < 0 || precond > 4) throw ArgError{"precond: 0 none, 1 Jacobi, 2 SSOR, 3 ILU(0), 4 multigrid"};
    if ((method == 1 || method == 4) && precond > 1)
        throw ArgError{"BiCGSTAB runs with no or the Jacobi preconditioner"};
    if (method == 2 && precond != 1) throw ArgError{"the mixed-precision CG uses the Jacobi preconditioner"};
    if (method == 5 && precond != 4) throw ArgError{"the multigrid CG takes precond 4 (multigrid)"};
    if (method != 5 && precond == 4) throw ArgError{"precond 4 (multigrid) goes with method 5"};
}
}  // namespace

extern "C" {

// method: 0 CG, 1 BiCGSTAB, 2 CG with FP32 recurrences (Jacobi), 3 GMRES(10),
// 4 BiCGSTAB with FP32 inner iterations in FP64 defect correction, 5 flexible
// CG with FP32 recurrences and FP64 reliable updates preconditioned by the
// aggregation-multigrid cycle (precond 4; omega = the smoother's Jacobi weight);
// precond: 0 none, 1 Jacobi (omega D^-1), 2 SSOR(omega), 3 ILU(0), 4 multigrid.
// x holds x0 on entry and the solution on return.  Returns 0, SYSU_ERR_INPUT
// for an argument error (checked before any device work), or SYSU_ERR_CUDA.
int sysu_csr_solve(int method, int precond, int n, const int *rowptr, const int *col, const double *val,
                   const double *b, double *x, int maxit, double eps, double omega, int *iters, double *res,
                   int *status) {
    try {
        check_method(method, precond);
        if (n < 1 || !rowptr || !col || !val || !b || !x) throw ArgError{"n >= 1 and non-null arrays required"};
        OwnedStream os;
        cudaStream_t st = os.st;
        {
            sysu::CsrDevice M;
            M.load(n, rowptr, col, val, st);
            sysu::DevBuf<double> db(n), dx(n);
            db.upload(b, n, st);
            dx.upload(x, n, st);
            sysu::KrylovWork w;
            sysu::DevBuf<sysu::SolveInfo> info(1);
            sysu::KrylovOpts o;
            o.maxit = maxit;
            o.eps = eps;
            o.omega = omega;
            o.jacobi = precond == 1;
            if (method == 0 && precond > 1) {
                sysu::pcg_solve(M.A, M.val.get(), db.get(), dx.get(), false, o, precond, w, info.get(), st);
            } else if (method == 0) {
                sysu::cg_solve(M.A, M.val.get(), db.get(), dx.get(), false, o, w, info.get(), st);
            } else if (method == 3) {
                sysu::gmres_solve(M.A, M.val.get(), db.get(), dx.get(), false, o, precond, 10, w, info.get(), st);
            } else if (method == 2) {
                sysu::DevBuf<float> v32(M.A.nnz);
                sysu::sell_to_fp32(M.A, M.val.get(), v32.get(), st);
                sysu::cg_solve_mixed(M.A, M.val.get(), v32.get(), db.get(), dx.get(), false, o, w, info.get(), st);
            } else if (method == 1) {
                const double *bb[1] = {db.get()};
                double *xx[1] = {dx.get()};
                sysu::bicgstab_solve(M.A, M.val.get(), 1, bb, xx, o, w, info.get(), st);
            } else if (method == 4) {
                sysu::bicgstab_solve_mixed(M.A, M.val.get(), db.get(), dx.get(), o, w, info.get(), st);
            } else {  // method 5 (check_method admits nothing else)
                sysu::DevBuf<float> v32(M.A.nnz);
                sysu::sell_to_fp32(M.A, M.val.get(), v32.get(), st);
                sysu::AggMultigrid mg;
                mg.omega = omega;
                mg.setup(M.A, M.pat, M.val.get(), 0.25, st);
                mg.refresh(M.val.get(), v32.get(), st);
                sysu::GnnPrecond fcg;
                fcg.bind(M.A, M.val.get(), v32.get(), st);
                fcg.attach_multigrid(&mg);
                o.inner_tol = 0.1;
                fcg.fcg(db.get(), dx.get(), false, o, false, info.get(), st);
                if (mg.err_flag(st)) throw sysu::CaseError{"multigrid: the coarsest level is singular"};
                sysu::SolveInfo h;
                info.download(&h, 1, st);
                dx.download(x, n, st);
                SYSU_CUDA(cudaStreamSynchronize(st));
                if (iters) *iters = h.iters[0];
                if (res) *res = h.res[0];
                if (status) *status = h.err ? sysu::DEV_BARRIER_TIMEOUT : h.status[0];
                return SYSU_OK;
            }
            sysu::SolveInfo h;
            info.download(&h, 1, st);
            dx.download(x, n, st);
            SYSU_CUDA(cudaStreamSynchronize(st));
            if (iters) *iters = h.iters[0];
            if (res) *res = h.res[0];
            if (status) *status = h.err ? sysu::DEV_BARRIER_TIMEOUT : h.status[0];
        }
        return SYSU_OK;
    } catch (const ArgError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_INPUT;
    } catch (const sysu::CaseError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_CUDA;
    }
}

int sysu_set_spmv_variant(int variant) {
    if (variant != 0 && variant != sysu::SPMV_RING && variant != sysu::SPMV_ASYNC && variant != sysu::SPMV_STAGE &&
        !(variant >= 11 && variant <= 99 && (variant % 10 == 1 || variant % 10 == 2 || variant % 10 == 4))) {
        g_csr_err = "sysu_set_spmv_variant: 0, 100, 200, 300 or 10 b + s with s in {1, 2, 4}";
        return SYSU_ERR_INPUT;
    }
    sysu::set_spmv_variant(variant);
    return SYSU_OK;
}

// y = A x for a host CSR matrix, on the GPU.
int sysu_csr_spmv(int n, const int *rowptr, const int *col, const double *val, const double *x, double *y) {
    try {
        OwnedStream os;
        cudaStream_t st = os.st;
        {
            sysu::CsrDevice M;
            M.load(n, rowptr, col, val, st);
            sysu::DevBuf<double> dx(n), dy(n);
            dx.upload(x, n, st);
            sysu::DevBuf<int> err(1);
            err.zero(st);
            if (sysu::spmv_variant() == sysu::SPMV_RING) sysu::spmv_ring(M.A, M.val.get(), dx.get(), dy.get(), err.get(), st);
            else sysu::spmv(M.A, M.val.get(), dx.get(), dy.get(), st);
            dy.download(y, n, st);
            int e = 0;
            err.download(&e, 1, st);
            SYSU_CUDA(cudaStreamSynchronize(st));
            if (e != 0) throw sysu::CaseError{"sysu_csr_spmv: a bounded wait of the ring SpMV gave up"};
        }
        return SYSU_OK;
    } catch (const ArgError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_INPUT;
    } catch (const sysu::CaseError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_CUDA;
    }
}

// Mean device ms of y = A x for a host CSR matrix (SELL-32 on the device) by the
// current standalone kernel form, the L2 flushed (256 MB read) before each of
// `reps` timed products; the same procedure as the solver's SpMV sweep.
int sysu_csr_spmv_timing(int n, const int *rowptr, const int *col, const double *val, int fp32, int reps,
                         double *ms) {
    try {
        if (n < 1 || !rowptr || !col || !val || !ms) throw ArgError{"n >= 1 and non-null arrays required"};
        if (reps < 1) reps = 1;
        OwnedStream os;
        cudaStream_t st = os.st;
        {
            sysu::CsrDevice M;
            M.load(n, rowptr, col, val, st);
            sysu::DevBuf<double> x64(n), y64(n);
            sysu::DevBuf<float> x32(n), y32(n), v32;
            sysu::DevBuf<unsigned char> flush((size_t)256 << 20);
            sysu::DevBuf<unsigned> sink(1);
            SYSU_CUDA(cudaMemsetAsync(flush.get(), 1, flush.size(), st));
            sysu::fill_sweep_x(n, x64.get(), x32.get(), st);
            if (fp32) {
                v32.alloc((size_t)M.A.nnz);
                sysu::sell_to_fp32(M.A, M.val.get(), v32.get(), st);
            }
            cudaEvent_t e0, e1;
            SYSU_CUDA(cudaEventCreate(&e0));
            SYSU_CUDA(cudaEventCreate(&e1));
            double total = 0.0;
            for (int k = 0; k < reps + 1; ++k) {
                sysu::l2_flush_read(flush.get(), flush.size(), sink.get(), st);
                SYSU_CUDA(cudaEventRecord(e0, st));
                if (fp32) sysu::spmv_stream32(M.A, v32.get(), x32.get(), y32.get(), st);
                else sysu::spmv_stream(M.A, M.val.get(), x64.get(), y64.get(), st);
                SYSU_CUDA(cudaEventRecord(e1, st));
                SYSU_CUDA(cudaEventSynchronize(e1));
                float t = 0.f;
                SYSU_CUDA(cudaEventElapsedTime(&t, e0, e1));
                if (k > 0) total += t;  // the first product warms up
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            *ms = total / reps;
        }
        return SYSU_OK;
    } catch (const ArgError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_INPUT;
    } catch (const sysu::CaseError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_CUDA;
    }
}

// Three systems with one sparsity pattern (rowptr, col) and their own values,
// solved by one batched BiCGSTAB + Jacobi launch.
int sysu_csr_bicgstab_batched3(int n, const int *rowptr, const int *col, const double *const *vals,
                               const double *const *b, double *const *x, int maxit, double eps, int *iters,
                               double *res, int *status) {
    try {
        if (!vals || !b || !x || n < 1 || !rowptr || !col) throw ArgError{"n >= 1 and non-null arrays required"};
        OwnedStream os;
        cudaStream_t st = os.st;
        {
            sysu::CsrDevice M;
            M.load(n, rowptr, col, vals[0], st);
            sysu::CsrDevice M1, M2;
            M1.pat = M.pat;
            M1.rp = M.rp;
            M1.cl = M.cl;
            M2.pat = M.pat;
            M2.rp = M.rp;
            M2.cl = M.cl;
            M1.reload_values(n, rowptr, col, vals[1], st);
            M2.reload_values(n, rowptr, col, vals[2], st);
            sysu::DevBuf<double> db[3], dx[3];
            for (int c = 0; c < 3; ++c) {
                db[c].alloc(n);
                dx[c].alloc(n);
                db[c].upload(b[c], n, st);
                dx[c].upload(x[c], n, st);
            }
            sysu::KrylovWork w;
            sysu::DevBuf<sysu::SolveInfo> info(1);
            sysu::KrylovOpts o;
            o.maxit = maxit;
            o.eps = eps;
            o.omega = 1.0;
            o.jacobi = true;
            const double *vv[3] = {M.val.get(), M1.val.get(), M2.val.get()};
            const double *bb[3] = {db[0].get(), db[1].get(), db[2].get()};
            double *xx[3] = {dx[0].get(), dx[1].get(), dx[2].get()};
            sysu::bicgstab_solve_multi(M.A, vv, bb, xx, o, w, info.get(), st);
            sysu::SolveInfo h;
            info.download(&h, 1, st);
            for (int c = 0; c < 3; ++c) dx[c].download(x[c], n, st);
            SYSU_CUDA(cudaStreamSynchronize(st));
            for (int c = 0; c < 3; ++c) {
                if (iters) iters[c] = h.iters[c];
                if (res) res[c] = h.res[c];
                if (status) status[c] = h.err ? sysu::DEV_BARRIER_TIMEOUT : h.status[c];
            }
        }
        return SYSU_OK;
    } catch (const ArgError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_INPUT;
    } catch (const sysu::CaseError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_CUDA;
    }
}

// Three right-hand sides b[c] of one matrix (the momentum form), x[c] x0 in and
// solution out: mixed 0 the FP64 batched BiCGSTAB + Jacobi, 1 the same with
// FP32 recurrences and FP64 residual replacement (inner_tol: the FP32 residual
// drop that triggers one); iters/res/status per component, refinements = the
// replacements summed over the components (0 for the FP64 form).
int sysu_csr_bicgstab3(int n, const int *rowptr, const int *col, const double *val, const double *const *b,
                       double *const *x, int mixed, int maxit, double eps, double omega, double inner_tol,
                       int *iters, double *res, int *status, int *refinements) {
    try {
        if (n < 1 || !rowptr || !col || !val || !b || !x) throw ArgError{"n >= 1 and non-null arrays required"};
        for (int c = 0; c < 3; ++c)
            if (!b[c] || !x[c]) throw ArgError{"b[0..2] and x[0..2] must be non-null"};
        if (mixed != 0 && mixed != 1) throw ArgError{"mixed: 0 FP64, 1 FP32 recurrences + FP64 replacement"};
        if (mixed && !(inner_tol > 0.0 && inner_tol < 1.0)) throw ArgError{"inner_tol must lie in (0, 1)"};
        if (maxit < 0 || !(eps > 0.0)) throw ArgError{"maxit >= 0 and eps > 0 required"};
        OwnedStream os;
        cudaStream_t st = os.st;
        {
            sysu::CsrDevice M;
            M.load(n, rowptr, col, val, st);
            sysu::DevBuf<double> db[3], dx[3];
            for (int c = 0; c < 3; ++c) {
                db[c].alloc(n);
                dx[c].alloc(n);
                db[c].upload(b[c], n, st);
                dx[c].upload(x[c], n, st);
            }
            sysu::KrylovWork w;
            sysu::DevBuf<sysu::SolveInfo> info(1);
            sysu::KrylovOpts o;
            o.maxit = maxit;
            o.eps = eps;
            o.omega = omega;
            o.jacobi = true;
            o.inner_tol = inner_tol;
            const double *bb[3] = {db[0].get(), db[1].get(), db[2].get()};
            double *xx[3] = {dx[0].get(), dx[1].get(), dx[2].get()};
            if (mixed) {
                sysu::Bicg3Mixed m;
                m.solve(M.A, M.val.get(), bb, xx, o, w, info.get(), st);
            } else {
                sysu::bicgstab_solve(M.A, M.val.get(), 3, bb, xx, o, w, info.get(), st);
            }
            sysu::SolveInfo h;
            info.download(&h, 1, st);
            for (int c = 0; c < 3; ++c) dx[c].download(x[c], n, st);
            SYSU_CUDA(cudaStreamSynchronize(st));
            for (int c = 0; c < 3; ++c) {
                if (iters) iters[c] = h.iters[c];
                if (res) res[c] = h.res[c];
                if (status) status[c] = h.err ? sysu::DEV_BARRIER_TIMEOUT : h.status[c];
            }
            if (refinements) *refinements = mixed ? h.refinements : 0;
        }
        return SYSU_OK;
    } catch (const ArgError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_INPUT;
    } catch (const sysu::CaseError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_CUDA;
    }
}

// Self-test of the device-side solve loops (CUDA graph WHILE nodes): *bodies =
// the number of loop bodies run when the stop flag is set after stop_at bodies
// (never, for stop_at <= 0) and the loop is bounded to `bound` bodies.
int sysu_graph_loop_selftest(int bound, int stop_at, int *bodies) {
    try {
        if (bound < 1 || !bodies) throw ArgError{"bound >= 1 and a non-null output required"};
        OwnedStream os;
        *bodies = sysu::graph_loop_selftest(bound, stop_at, os.st);
        return SYSU_OK;
    } catch (const ArgError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_INPUT;
    } catch (const sysu::CaseError &e) {
        g_csr_err = e.msg;
        return SYSU_ERR_CUDA;
    }
}

const char *sysu_csr_last_error(void) { return g_csr_err.c_str(); }

// Assembled matrix of a solver ("mom", "p", "scalar", "solid") as CSR with the
// diagonal first in each row.  rowptr: n+1, col/val: the true entry count
// (sysu_solver_info out[5], or the solid's own count).  Returns the entry count.
long sysu_solver_matrix(sysu_solver *s, const char *which, int *rowptr, int *col, double *val) {
    if (!s || !which) return -1;
    try {
        sysu::SimpleSolver &S = *s->impl;
        std::string w(which);
        const sysu::DomainDev *d = &S.fd;
        const sysu::DevBuf<double> *v = nullptr;
        if (w == "mom") v = &S.f.Amom;
        else if (w == "p") v = &S.f.Ap;
        else if (w == "scalar") v = &S.f.As;
        else if (w == "solid" && S.cs.has_solid) { d = &S.sd; v = &S.s.As; }
        else return -1;
        const sysu::SellPattern &p = d->pat;
        if (!rowptr) return p.nnz_true;
        std::vector<double> h(p.nnz);
        v->download(h.data(), p.nnz, S.st);
        SYSU_CUDA(cudaStreamSynchronize(S.st));
        long k = 0;
        rowptr[0] = 0;
        for (int i = 0; i < p.n; ++i) {
            for (int j = 0; j < p.row_len[i]; ++j) {
                col[k] = p.col[p.pos(i, j)];
                val[k] = h[p.pos(i, j)];
                ++k;
            }
            rowptr[i + 1] = (int)k;
        }
        return k;
    } catch (const sysu::CaseError &e) {
        g_csr_err = e.msg;
        return -1;
    }
}

}  // extern "C"
