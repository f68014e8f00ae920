// C ABI of the learned preconditioner (include/sysu_cfd.h, sysu_gnn_*): a host
// CSR matrix on the device, the network, its training ring and flexible CG.
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sysu_cfd.h"
#include "csr_device.hpp"
#include "gnn.hpp"

struct sysu_gnn {
    cudaStream_t st = nullptr;
    sysu::CsrDevice M;
    sysu::DevBuf<float> val32;
    sysu::AggMultigrid mg;  // declared before net: net refers to it and goes first
    sysu::GnnPrecond net;
    sysu::DevBuf<double> v0, v1;
    sysu::DevBuf<sysu::SolveInfo> info;
};

namespace {
thread_local std::string g_gnn_err;

template <class F>
int guarded(F f) {
    try {
        f();
        return SYSU_OK;
    } catch (const sysu::CaseError &e) {
        g_gnn_err = e.msg;
        return SYSU_ERR_CUDA;
    }
}
}  // namespace

extern "C" {

int sysu_gnn_num_params(void) { return sysu::GNN_NPARAM; }

int sysu_gnn_create(int n, const int *rowptr, const int *col, const double *val, int capacity, sysu_gnn **out) {
    if (!out || n <= 0 || !rowptr || !col || !val || capacity <= 0) {
        g_gnn_err = "sysu_gnn_create: bad arguments";
        return SYSU_ERR_INPUT;
    }
    *out = nullptr;
    sysu_gnn *g = new sysu_gnn;
    int rc = guarded([&] {
        SYSU_CUDA(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking));
        g->M.load(n, rowptr, col, val, g->st);
        g->val32.alloc(g->M.A.nnz);
        sysu::sell_to_fp32(g->M.A, g->M.val.get(), g->val32.get(), g->st);
        g->net.set_capacity(capacity);
        g->net.bind(g->M.A, g->M.val.get(), g->val32.get(), g->st);
        g->v0.alloc(n);
        g->v1.alloc(n);
        g->info.alloc(1);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
    if (rc != SYSU_OK) {
        sysu_gnn_free(g);
        return rc;
    }
    *out = g;
    return SYSU_OK;
}

void sysu_gnn_free(sysu_gnn *g) {
    if (!g) return;
    cudaStream_t st = g->st;
    if (st) cudaStreamSynchronize(st);
    delete g;
    if (st) cudaStreamDestroy(st);
}

int sysu_gnn_set_values(sysu_gnn *g, const int *rowptr, const int *col, const double *val) {
    if (!g || !rowptr || !col || !val) return SYSU_ERR_INPUT;
    return guarded([&] {
        g->M.reload_values(g->net.n(), rowptr, col, val, g->st);
        sysu::sell_to_fp32(g->M.A, g->M.val.get(), g->val32.get(), g->st);
        g->net.refresh(g->st);
        if (g->net.multigrid()) g->mg.refresh(g->M.val.get(), g->val32.get(), g->st);
    });
}

int sysu_gnn_init_params(sysu_gnn *g, unsigned long long seed) {
    if (!g) return SYSU_ERR_INPUT;
    return guarded([&] {
        g->net.init_params(seed, g->st);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int sysu_gnn_set_params(sysu_gnn *g, const float *p, int np) {
    if (!g || !p || np != sysu::GNN_NPARAM) {
        g_gnn_err = "sysu_gnn_set_params: need sysu_gnn_num_params() values";
        return SYSU_ERR_INPUT;
    }
    return guarded([&] {
        g->net.set_params(p, g->st);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int sysu_gnn_get_params(sysu_gnn *g, float *p, int np) {
    if (!g || !p || np != sysu::GNN_NPARAM) {
        g_gnn_err = "sysu_gnn_get_params: need sysu_gnn_num_params() values";
        return SYSU_ERR_INPUT;
    }
    return guarded([&] { g->net.get_params(p, g->st); });
}

int sysu_gnn_apply(sysu_gnn *g, const double *r, double *z) {
    if (!g || !r || !z) return SYSU_ERR_INPUT;
    return guarded([&] {
        int n = g->net.n();
        g->v0.upload(r, n, g->st);
        g->net.apply(g->v0.get(), g->v1.get(), g->st);
        g->v1.download(z, n, g->st);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int sysu_gnn_add_pair(sysu_gnn *g, const double *r, const double *e) {
    if (!g || !r || !e) return SYSU_ERR_INPUT;
    return guarded([&] {
        int n = g->net.n();
        g->v0.upload(r, n, g->st);
        g->v1.upload(e, n, g->st);
        g->net.add_pair(g->v0.get(), g->v1.get(), g->st);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int sysu_gnn_loss_grad(sysu_gnn *g, int k, int loss_kind, double *loss, float *grad, int np) {
    if (!g || !loss || !grad || np != sysu::GNN_NPARAM || (loss_kind != 0 && loss_kind != 1)) return SYSU_ERR_INPUT;
    return guarded([&] {
        g->net.loss_kind = loss_kind;
        g->net.loss_grad(k, loss, grad, g->st);
    });
}

int sysu_gnn_train(sysu_gnn *g, int steps, double lr, int loss_kind, double *losses) {
    if (!g || steps < 0 || (loss_kind != 0 && loss_kind != 1)) return SYSU_ERR_INPUT;
    return guarded([&] {
        g->net.loss_kind = loss_kind;
        int np = g->net.pairs();
        if (np == 0) throw sysu::CaseError{"sysu_gnn_train: no training pairs"};
        for (int s = 0; s < steps; ++s) g->net.train_step(s % np, lr, g->st);
        if (losses && steps > 0) {
            std::vector<double> l;
            g->net.last_losses(l, steps, g->st);
            std::memcpy(losses, l.data(), l.size() * sizeof(double));
        }
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int sysu_gnn_fcg(sysu_gnn *g, const double *b, double *x, int x0_zero, int maxit, double eps, double inner_tol,
                 int use_gnn, int stall_max, int *iters, double *res, int *status, int *fallback_at,
                 int *refinements, double *seconds) {
    if (!g || !b || !x || maxit < 0 || !(eps > 0.0) || !(inner_tol > 0.0 && inner_tol < 1.0)) return SYSU_ERR_INPUT;
    return guarded([&] {
        int n = g->net.n();
        g->v0.upload(b, n, g->st);
        if (!x0_zero) g->v1.upload(x, n, g->st);
        sysu::KrylovOpts o;
        o.maxit = maxit;
        o.eps = eps;
        o.inner_tol = inner_tol;
        g->net.stall_max = stall_max > 0 ? stall_max : 30;
        cudaEvent_t e0, e1;
        SYSU_CUDA(cudaEventCreate(&e0));
        SYSU_CUDA(cudaEventCreate(&e1));
        SYSU_CUDA(cudaEventRecord(e0, g->st));
        g->net.fcg(g->v0.get(), g->v1.get(), x0_zero != 0, o, use_gnn != 0, g->info.get(), g->st);
        SYSU_CUDA(cudaEventRecord(e1, g->st));
        g->v1.download(x, n, g->st);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        sysu::FcgState f = g->net.last_state(g->st);
        if (iters) *iters = f.iters;
        if (res) *res = f.res;
        if (status) *status = f.status;
        if (fallback_at) *fallback_at = f.fallback_at;
        if (refinements) *refinements = f.refinements;
        if (seconds) *seconds = ms * 1e-3;
    });
}

int sysu_gnn_hidden(sysu_gnn *g, const double *r, int layer, float *h) {
    if (!g || !r || !h) return SYSU_ERR_INPUT;
    return guarded([&] {
        g->v0.upload(r, g->net.n(), g->st);
        g->net.hidden(g->v0.get(), layer, h, g->st);
    });
}

int sysu_gnn_time_apply(sysu_gnn *g, const double *r, int reps, int fwd_per_sm, double *ms) {
    if (!g || !r || !ms) return SYSU_ERR_INPUT;
    return guarded([&] {
        g->v0.upload(r, g->net.n(), g->st);
        if (fwd_per_sm != g->net.fwd_per_sm) {
            g->net.fwd_per_sm = fwd_per_sm;
            g->net.bind(g->M.A, g->M.val.get(), g->val32.get(), g->st);
        }
        *ms = g->net.time_apply(g->v0.get(), reps, g->st);
    });
}

int sysu_gnn_set_multigrid(sysu_gnn *g, int on, double theta, double omega, double gamma, int *levels, int *rows,
                           int max_levels) {
    if (!g || (on && (!(theta > 0.0 && theta < 1.0) || !(omega > 0.0 && omega < 2.0) || !(gamma > 0.0 && gamma <= 4.0)))) {
        g_gnn_err = "sysu_gnn_set_multigrid: theta in (0, 1), omega in (0, 2), gamma in (0, 4]";
        return SYSU_ERR_INPUT;
    }
    return guarded([&] {
        g->net.attach_multigrid(nullptr);
        g->net.skip = 1.0f;  // the network as the whole preconditioner
        if (!on) return;
        g->net.skip = (float)omega;  // the cycle's post-smoother: zero decoder = its Jacobi step
        g->mg.omega = omega;
        g->mg.gamma = gamma;
        g->mg.setup(g->M.A, g->M.pat, g->M.val.get(), theta, g->st);
        g->mg.refresh(g->M.val.get(), g->val32.get(), g->st);
        g->net.attach_multigrid(&g->mg);
        if (g->mg.err_flag(g->st)) throw sysu::CaseError{"multigrid: the coarsest level is singular"};
        if (levels) *levels = g->mg.levels();
        if (rows)
            for (int l = 0; l < g->mg.levels() && l < max_levels; ++l) rows[l] = g->mg.level_rows(l);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int sysu_gnn_mg_apply(sysu_gnn *g, const double *r, double *z, int use_gnn) {
    if (!g || !r || !z) return SYSU_ERR_INPUT;
    return guarded([&] {
        int n = g->net.n();
        g->v0.upload(r, n, g->st);
        g->net.apply_mg(g->v0.get(), g->v1.get(), use_gnn != 0, g->st);
        g->v1.download(z, n, g->st);
        SYSU_CUDA(cudaStreamSynchronize(g->st));
    });
}

const char *sysu_gnn_last_error(void) { return g_gnn_err.c_str(); }

}  // extern "C"
