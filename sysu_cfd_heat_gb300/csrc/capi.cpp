// C ABI of libsysucfd.so (declared in include/sysu_cfd.h).
#include "../../include/sysu_cfd.h"

#include <algorithm>
#include <cstring>
#include <exception>
#include <string>

#include <fstream>
#include <limits>
#include "batch.hpp"
#include "handles.hpp"
#include "output.hpp"

namespace {
thread_local std::string g_err;

int set_err(int code, const std::string &m) {
    g_err = m;
    return code;
}

template <class F>
int guarded(F &&fn) {
    try {
        return fn();
    } catch (const sysu::CaseError &e) {
        bool cuda = e.msg.find("cuda") != std::string::npos || e.msg.find("CUDA") != std::string::npos;
        return set_err(cuda ? SYSU_ERR_CUDA : SYSU_ERR_INPUT, e.msg);
    } catch (const std::exception &e) {
        return set_err(SYSU_ERR_INPUT, e.what());
    }
}

template <class T>
long copy_vec(const std::vector<T> &v, void *out, long nbytes) {
    long sz = (long)(v.size() * sizeof(T));
    if (out && nbytes > 0) std::memcpy(out, v.data(), (size_t)std::min(sz, nbytes));
    return sz;
}

sysu::EqOpts *eq_of(sysu::SolverOptions &o, const std::string &k) {
    if (k == "mom") return &o.mom;
    if (k == "p") return &o.p;
    if (k == "ke") return &o.ke;
    if (k == "t") return &o.t;
    if (k == "ts") return &o.ts;
    return nullptr;
}
}  // namespace

extern "C" {

const char *sysu_last_error(void) { return g_err.c_str(); }
int sysu_version(void) { return 1; }

int sysu_case_load(const char *param_path, sysu_case **out) {
    if (!param_path || !out) return set_err(SYSU_ERR_INPUT, "null argument");
    *out = nullptr;
    return guarded([&] {
        sysu_case *c = new sysu_case;
        try {
            c->cs.params = sysu::parse_params(param_path);
            std::string grid = c->cs.params.gridfile;
            sysu::RawMesh raw;
            try {
                raw = sysu::read_msh(grid);
            } catch (const sysu::CaseError &) {
                std::string pp(param_path);
                size_t slash = pp.find_last_of('/');
                if (slash == std::string::npos || (!grid.empty() && grid[0] == '/')) throw;
                raw = sysu::read_msh(pp.substr(0, slash + 1) + grid);
            }
            sysu::build_case(raw, c->cs);
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
        return SYSU_OK;
    });
}

void sysu_case_free(sysu_case *c) { delete c; }

int sysu_case_info(const sysu_case *c, long *out, int n) {
    if (!c || !out) return set_err(SYSU_ERR_INPUT, "null argument");
    long v[12] = {c->cs.fluid.nc, c->cs.fluid.nf, c->cs.fluid.nb, c->cs.fluid.nv, c->cs.fluid.ncb,
                  c->cs.solid.nc, c->cs.solid.nf, c->cs.solid.nb, c->cs.solid.nv, c->cs.solid.ncb,
                  c->cs.has_solid ? 1 : 0, c->cs.coupled_rid};
    for (int i = 0; i < n && i < 12; ++i) out[i] = v[i];
    return SYSU_OK;
}

long sysu_case_array(const sysu_case *c, const char *name, void *out, long nbytes) {
    if (!c || !name) return -1;
    std::string nm(name);
    const sysu::Domain *d = &c->cs.fluid;
    if (nm.rfind("solid_", 0) == 0) {
        if (!c->cs.has_solid) return -1;
        d = &c->cs.solid;
        nm = nm.substr(6);
    }
    if (nm == "cell_vol") return copy_vec(d->cell_vol, out, nbytes);
    if (nm == "cell_x") return copy_vec(d->cell_x, out, nbytes);
    if (nm == "cell_nface") return copy_vec(d->cell_nface, out, nbytes);
    if (nm == "cell_face") return copy_vec(d->cell_face, out, nbytes);
    if (nm == "cell_nbr") return copy_vec(d->cell_nbr, out, nbytes);
    if (nm == "cell_rid") return copy_vec(d->cell_rid, out, nbytes);
    if (nm == "cell_vert") return copy_vec(d->cell_vert, out, nbytes);
    if (nm == "face_x") return copy_vec(d->face_x, out, nbytes);
    if (nm == "face_n") return copy_vec(d->face_n, out, nbytes);
    if (nm == "face_area") return copy_vec(d->face_area, out, nbytes);
    if (nm == "face_lambda") return copy_vec(d->face_lambda, out, nbytes);
    if (nm == "face_rlencos") return copy_vec(d->face_rlencos, out, nbytes);
    if (nm == "face_xpac") return copy_vec(d->face_xpac, out, nbytes);
    if (nm == "face_xnac") return copy_vec(d->face_xnac, out, nbytes);
    if (nm == "face_c1") return copy_vec(d->face_c1, out, nbytes);
    if (nm == "face_c2") return copy_vec(d->face_c2, out, nbytes);
    if (nm == "face_bnd") return copy_vec(d->face_bnd, out, nbytes);
    if (nm == "face_vert") return copy_vec(d->face_vert, out, nbytes);
    if (nm == "bnd_face") return copy_vec(d->bnd_face, out, nbytes);
    if (nm == "bnd_rid") return copy_vec(d->bnd_rid, out, nbytes);
    if (nm == "bnd_distance") return copy_vec(d->bnd_distance, out, nbytes);
    if (nm == "vert") return copy_vec(d->vert, out, nbytes);
    return -1;
}

int sysu_solver_create(const char *param_path, sysu_solver **out) {
    if (!param_path || !out) return set_err(SYSU_ERR_INPUT, "null argument");
    *out = nullptr;
    return guarded([&] {
        sysu_solver *s = new sysu_solver{nullptr};
        try {
            s->impl = new sysu::SimpleSolver(param_path);
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
        return SYSU_OK;
    });
}

void sysu_solver_destroy(sysu_solver *s) {
    if (!s) return;
    try {
        delete s->impl;
    } catch (...) {
    }
    delete s;
}

int sysu_solver_info(sysu_solver *s, long *out, int n) {
    if (!s || !out) return set_err(SYSU_ERR_INPUT, "null argument");
    sysu::SimpleSolver &S = *s->impl;
    long v[6] = {S.fd.nc, S.fd.nf, S.fd.B, S.cs.has_solid ? S.sd.nc : 0, S.fd.A.nnz, S.fd.A.nnz_true};
    for (int i = 0; i < n && i < 6; ++i) out[i] = v[i];
    return SYSU_OK;
}

int sysu_solver_set_option(sysu_solver *s, const char *key, double value) {
    if (!s || !key) return set_err(SYSU_ERR_INPUT, "null argument");
    sysu::SolverOptions &o = s->impl->opt;
    std::string k(key);
    if (k == "rtc") {
        o.mom.eps = o.p.eps = o.ke.eps = o.t.eps = o.ts.eps = value;
        return SYSU_OK;
    }
    if (k == "mom_batched") { o.mom_batched = value != 0.0; return SYSU_OK; }
    if (k == "graph_loops") { o.graph_loops = value != 0.0; return SYSU_OK; }
    if (k == "sm_cap") { s->impl->kw.sm_cap = std::max(0, (int)value); return SYSU_OK; }
    if (k == "spmv_variant") { sysu::set_spmv_variant((int)value); return SYSU_OK; }
    if (k == "convection") {
        if (value != 0.0 && value != 1.0) return set_err(SYSU_ERR_INPUT, "convection: 0 upwind + deferred correction, 1 hybrid");
        o.convection = (int)value;
        return SYSU_OK;
    }
    if (k == "gradient") {
        if (value != 0.0 && value != 1.0) return set_err(SYSU_ERR_INPUT, "gradient: 0 Green-Gauss, 1 least squares");
        try {
            s->impl->set_gradient_scheme((int)value);
        } catch (const sysu::CaseError &e) {
            return set_err(SYSU_ERR_CUDA, e.msg);
        }
        return SYSU_OK;
    }
    if (k == "scalars_batched") {
        const sysu::Params &pp = s->impl->cs.params;
        if (value != 0.0 && (pp.tur_model != 1 || !pp.solve_energy))
            return set_err(SYSU_ERR_INPUT, "scalars_batched needs turbulence ke and energy on");
        if (value != 0.0 && (o.ke.kind != sysu::SK_BICGSTAB || o.t.kind != sysu::SK_BICGSTAB ||
                             o.ke.precond > sysu::PK_JACOBI || o.t.precond > sysu::PK_JACOBI))
            return set_err(SYSU_ERR_INPUT, "scalars_batched runs k, eps and T with BiCGSTAB + Jacobi");
        if (value != 0.0 && (o.ke.mixed || o.t.mixed))
            return set_err(SYSU_ERR_INPUT, "scalars_batched solves k, eps and T in FP64; turn ke.mixed / t.mixed off first");
        o.scalars_batched = value != 0.0;
        return SYSU_OK;
    }
    if (k == "reference_solvers") {
        if (value != 0.0) o.reference_solvers();
        else o.default_solvers();
        // perfect gas: p' is not symmetric, the reference solves it with GMRES
        // (navier_pressure.cpp:28-31)
        if (s->impl->cs.params.density_model == 1) o.p.kind = value != 0.0 ? sysu::SK_GMRES : sysu::SK_BICGSTAB;
        return SYSU_OK;
    }
    if (k == "solid_source") { o.solid_source = value; return SYSU_OK; }
    if (k == "fatal_checks") { o.fatal_checks = value != 0.0; return SYSU_OK; }
    if (k == "timing") { o.timing = value != 0.0; return SYSU_OK; }
    if (k == "output") { o.output = value != 0.0; return SYSU_OK; }
    if (k == "profile_phases") {
        return guarded([&] {
            sysu::SimpleSolver &S = *s->impl;
            o.profile_phases = value != 0.0;
            if (o.profile_phases && !S.phase_ts.get()) {
                S.phase_ts.alloc(4 * 64);
                S.phase_ts.zero(S.st);
            }
            S.kw.phase_ts = o.profile_phases ? S.phase_ts.get() : nullptr;
            return SYSU_OK;
        });
    }
    size_t dot = k.find('.');
    if (dot != std::string::npos) {
        sysu::EqOpts *e = eq_of(o, k.substr(0, dot));
        std::string f = k.substr(dot + 1);
        if (e) {
            if (f == "eps") { e->eps = value; return SYSU_OK; }
            if (f == "maxit") { e->maxit = (int)value; return SYSU_OK; }
            if (f == "omega") { e->omega = value; return SYSU_OK; }
            if (f == "mixed") {
                if (value != 0.0 && e->kind == sysu::SK_GMRES)
                    return set_err(SYSU_ERR_INPUT, "mixed precision is available for CG and BiCGSTAB solves");
                if (value != 0.0 && e->kind == sysu::SK_CG && e->precond != sysu::PK_JACOBI && e->precond != sysu::PK_AMG)
                    return set_err(SYSU_ERR_INPUT, "the mixed-precision CG uses the Jacobi preconditioner");
                if (value != 0.0 && o.scalars_batched && (e == &o.ke || e == &o.t))
                    return set_err(SYSU_ERR_INPUT, "scalars_batched solves k, eps and T in FP64; turn it off first");
                e->mixed = value != 0.0;
                return SYSU_OK;
            }
            if (f == "inner_tol") {
                if (!(value > 0.0 && value < 1.0)) return set_err(SYSU_ERR_INPUT, "inner_tol must lie in (0, 1)");
                e->inner_tol = value;
                return SYSU_OK;
            }
            if (f == "kind") {
                int kind = (int)value;
                if (kind != sysu::SK_CG && kind != sysu::SK_BICGSTAB && kind != sysu::SK_GMRES)
                    return set_err(SYSU_ERR_INPUT, "kind: 0 CG, 1 BiCGSTAB, 2 GMRES");
                if (kind == sysu::SK_CG && e == &o.mom) return set_err(SYSU_ERR_INPUT, "momentum matrix is not symmetric");
                if (kind == sysu::SK_CG && e == &o.p && s->impl->cs.params.density_model == 1)
                    return set_err(SYSU_ERR_INPUT, "the perfect-gas p' matrix is not symmetric");
                if (kind == sysu::SK_BICGSTAB && e->precond > sysu::PK_JACOBI)
                    return set_err(SYSU_ERR_INPUT, "BiCGSTAB runs with no or the Jacobi preconditioner");
                if (kind == sysu::SK_GMRES) e->mixed = 0;
                e->kind = kind;
                return SYSU_OK;
            }
            if (f == "precond") {
                int pc = (int)value;
                if (pc < sysu::PK_NONE || pc > sysu::PK_AMG)
                    return set_err(SYSU_ERR_INPUT, "precond: 0 none, 1 Jacobi, 2 SSOR, 3 ILU(0), 4 multigrid (p')");
                if (pc == sysu::PK_AMG && (e != &o.p || e->kind != sysu::SK_CG))
                    return set_err(SYSU_ERR_INPUT, "the multigrid preconditioner is for the p' CG");
                if (pc > sysu::PK_JACOBI && e->kind == sysu::SK_BICGSTAB)
                    return set_err(SYSU_ERR_INPUT, "BiCGSTAB runs with no or the Jacobi preconditioner");
                if (pc != sysu::PK_JACOBI && pc != sysu::PK_AMG && e->mixed)
                    return set_err(SYSU_ERR_INPUT, "the mixed-precision CG uses the Jacobi preconditioner");
                if (e->learned && pc != sysu::PK_JACOBI && pc != sysu::PK_AMG)
                    return set_err(SYSU_ERR_INPUT, "the learned form runs with the Jacobi or multigrid preconditioner");
                e->precond = pc;
                return SYSU_OK;
            }
            if (f == "restart") {
                int m = (int)value;
                if (m < 1 || m > sysu::GMRES_MAX_RESTART) return set_err(SYSU_ERR_INPUT, "restart: 1..30");
                e->restart = m;
                return SYSU_OK;
            }
            if (f == "learned") {
                if (value != 0.0 && (e != &o.p || e->kind != sysu::SK_CG ||
                                     (e->precond != sysu::PK_JACOBI && e->precond != sysu::PK_AMG)))
                    return set_err(SYSU_ERR_INPUT, "the learned preconditioner is for the p' CG (Jacobi or multigrid mode)");
                e->learned = value != 0.0;
                return SYSU_OK;
            }
            if (f == "learn_iters") { e->learn_iters = std::max(0, (int)value); return SYSU_OK; }
            if (f == "learn_reset") {
                // start the learned form over: fresh network, empty pair ring, new training window
                if (e != &o.p) return set_err(SYSU_ERR_INPUT, "learn_reset is a p' option");
                return guarded([&] {
                    sysu::SimpleSolver &S = *s->impl;
                    S.p_solves = 0;
                    for (sysu::GnnPrecond *g : {&S.gnn, &S.gnn_c}) {
                        if (!g->bound()) continue;
                        g->init_params(20261203ULL, S.st);
                        g->reset_adam(S.st);
                        g->clear_pairs();
                    }
                    return SYSU_OK;
                });
            }
            if (f == "mg_theta") {
                if (!(value > 0.0 && value < 1.0)) return set_err(SYSU_ERR_INPUT, "mg_theta: strength threshold in (0, 1)");
                e->mg_theta = value;
                return SYSU_OK;
            }
            if (f == "mg_omega") {
                if (!(value > 0.0 && value < 2.0)) return set_err(SYSU_ERR_INPUT, "mg_omega: Jacobi weight in (0, 2)");
                e->mg_omega = value;
                return SYSU_OK;
            }
            if (f == "mg_gamma") {
                if (!(value > 0.0 && value <= 4.0)) return set_err(SYSU_ERR_INPUT, "mg_gamma: correction scale in (0, 4]");
                e->mg_gamma = value;
                return SYSU_OK;
            }
            if (f == "mg_persistent") { e->mg_persistent = value != 0.0; return SYSU_OK; }
            if (f == "learn_level") {
                if (value < 0.0 || value > 15.0) return set_err(SYSU_ERR_INPUT, "learn_level: multigrid level 0..15");
                e->learn_level = (int)value;
                return SYSU_OK;
            }
            if (f == "learn_steps") { e->learn_steps = std::max(0, (int)value); return SYSU_OK; }
            if (f == "learn_lr") { e->learn_lr = value; return SYSU_OK; }
            if (f == "learn_kind") {
                if (value != 0.0 && value != 1.0) return set_err(SYSU_ERR_INPUT, "learn_kind: 0 energy norm, 1 residual norm");
                e->learn_kind = (int)value;
                s->impl->gnn.loss_kind = e->learn_kind;
                return SYSU_OK;
            }
        }
    }
    return set_err(SYSU_ERR_INPUT, "unknown option " + k);
}

int sysu_solver_get_option(sysu_solver *s, const char *key, double *value) {
    if (!s || !key || !value) return set_err(SYSU_ERR_INPUT, "null argument");
    sysu::SolverOptions &o = s->impl->opt;
    std::string k(key);
    if (k == "mom_batched") { *value = o.mom_batched; return SYSU_OK; }
    if (k == "graph_loops") { *value = o.graph_loops; return SYSU_OK; }
    if (k == "scalars_batched") { *value = o.scalars_batched; return SYSU_OK; }
    if (k == "gradient") { *value = s->impl->gradient_scheme; return SYSU_OK; }
    if (k == "convection") { *value = o.convection; return SYSU_OK; }
    if (k == "sm_cap") { *value = s->impl->kw.sm_cap; return SYSU_OK; }
    if (k == "solid_source") { *value = o.solid_source; return SYSU_OK; }
    if (k == "fatal_checks") { *value = o.fatal_checks; return SYSU_OK; }
    if (k == "timing") { *value = o.timing; return SYSU_OK; }
    if (k == "output") { *value = o.output; return SYSU_OK; }
    if (k == "profile_phases") { *value = o.profile_phases; return SYSU_OK; }
    size_t dot = k.find('.');
    if (dot != std::string::npos) {
        sysu::EqOpts *e = eq_of(o, k.substr(0, dot));
        std::string f = k.substr(dot + 1);
        if (e) {
            if (f == "eps") { *value = e->eps; return SYSU_OK; }
            if (f == "maxit") { *value = e->maxit; return SYSU_OK; }
            if (f == "omega") { *value = e->omega; return SYSU_OK; }
            if (f == "kind") { *value = e->kind; return SYSU_OK; }
            if (f == "mixed") { *value = e->mixed; return SYSU_OK; }
            if (f == "precond") { *value = e->precond; return SYSU_OK; }
            if (f == "restart") { *value = e->restart; return SYSU_OK; }
            if (f == "inner_tol") { *value = e->inner_tol; return SYSU_OK; }
            if (f == "learned") { *value = e->learned; return SYSU_OK; }
            if (f == "learn_iters") { *value = e->learn_iters; return SYSU_OK; }
            if (f == "mg_theta") { *value = e->mg_theta; return SYSU_OK; }
            if (f == "mg_omega") { *value = e->mg_omega; return SYSU_OK; }
            if (f == "mg_gamma") { *value = e->mg_gamma; return SYSU_OK; }
            if (f == "mg_persistent") { *value = e->mg_persistent; return SYSU_OK; }
            if (f == "learn_level") { *value = e->learn_level; return SYSU_OK; }
            if (f == "learn_steps") { *value = e->learn_steps; return SYSU_OK; }
            if (f == "learn_lr") { *value = e->learn_lr; return SYSU_OK; }
            if (f == "learn_kind") { *value = e->learn_kind; return SYSU_OK; }
        }
    }
    if (k == "p.learned_solves") { *value = s->impl->p_solves; return SYSU_OK; }
    return set_err(SYSU_ERR_INPUT, "unknown option " + k);
}

static int run_iterations(sysu_solver *s, int n, int *done) {
    sysu::SimpleSolver &S = *s->impl;
    int k = 0;
    for (; k < n; ++k) {
        std::string msg = S.outer_iteration();
        if (!msg.empty()) {
            if (done) *done = k + 1;
            return set_err(SYSU_ERR_SOLVE, msg);
        }
        double resmax = 0.0;  // vec_max starts from 0 (tools.cpp:81-87)
        for (double r : S.Residual) resmax = resmax > r ? resmax : r;
        if (S.cs.params.steady && resmax < S.cs.params.residual_steady) {
            ++k;
            break;
        }
    }
    if (done) *done = k;
    return SYSU_OK;
}

int sysu_solver_iterate(sysu_solver *s, int n, int *done) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] { return run_iterations(s, n, done); });
}

// The transient NSSolve (navier.cpp:20-90): per time step SaveTransientOldData,
// then outer iterations until max(Residual) < 1e-4 or it fell 1000-fold since the
// step's first iteration (at most MaxOuterStep-1), VolumnAverage, advance time.
static int run_transient(sysu_solver *s, int *done) {
    sysu::SimpleSolver &S = *s->impl;
    const sysu::Params &p = S.cs.params;
    const std::string dir = S.case_dir;
    if (S.opt.output) sysu::write_tot_header(dir + "/tot.dat");
    double cur_time = p.dt;
    int total = 0;
    for (int step = 1; step <= p.max_step; ++step) {
        S.save_transient_old_data();
        double resmax0 = 0.0;
        int iter = 1;
        for (; iter < p.max_outer_step; ++iter) {
            std::string msg = S.outer_iteration();
            ++total;
            if (!msg.empty()) {
                if (done) *done = total;
                return set_err(SYSU_ERR_SOLVE, msg);
            }
            double resmax = 0.0;
            for (double r : S.Residual) resmax = resmax > r ? resmax : r;
            if (iter == 1) resmax0 = resmax;
            if (resmax < 1.e-4 || resmax0 / (resmax + 1.e-16) > 1000.) break;
        }
        if (S.opt.output) S.volume_average(dir, cur_time, iter);
        if (cur_time >= p.total_time) break;
        cur_time += p.dt;
    }
    if (S.opt.output) S.output(dir);
    if (done) *done = total;
    return SYSU_OK;
}

int sysu_solver_nssolve(sysu_solver *s, int *done) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    sysu::SimpleSolver &S = *s->impl;
    if (!S.cs.params.steady) return guarded([&] { return run_transient(s, done); });
    if (!S.opt.output) return guarded([&] { return run_iterations(s, S.cs.params.max_outer_step - 1, done); });
    // navier.cpp:13-97 for a steady case, with its writers: tot.dat header
    // (constructor), Output() every noutput iterations and at the end,
    // VolumnAverage(cur_time = DBL_MAX, iter) after the loop.
    return guarded([&] {
        const std::string dir = S.case_dir;
        sysu::write_tot_header(dir + "/tot.dat");
        const int last = S.cs.params.max_outer_step;
        const int nout = S.cs.params.noutput > 0 ? S.cs.params.noutput : 1;
        int iter = 1;
        for (; iter < last; ++iter) {
            std::string msg = S.outer_iteration();
            if (!msg.empty()) {
                if (done) *done = iter;
                return set_err(SYSU_ERR_SOLVE, msg);
            }
            if ((iter - 1) % nout == 0) S.output(dir);
            double resmax = 0.0;
            for (double r : S.Residual) resmax = resmax > r ? resmax : r;
            if (S.cs.params.steady && resmax < S.cs.params.residual_steady) break;
        }
        if (done) *done = iter < last ? iter : last - 1;
        S.volume_average(dir, std::numeric_limits<double>::max(), iter);
        S.output(dir);
        return SYSU_OK;
    });
}

int sysu_solver_output(sysu_solver *s, const char *dir) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        s->impl->output(dir ? std::string(dir) : s->impl->case_dir);
        return SYSU_OK;
    });
}

int sysu_solver_volume_average(sysu_solver *s, const char *dir, double t, int out_iter) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        std::string d = dir ? std::string(dir) : s->impl->case_dir;
        std::ifstream probe(d + "/tot.dat");
        if (!probe.good()) sysu::write_tot_header(d + "/tot.dat");
        s->impl->volume_average(d, t, out_iter);
        return SYSU_OK;
    });
}

int sysu_case_write_tecplot(const sysu_case *c, const char *path, int nfields, const char *const *names,
                            const double *const *arrays) {
    if (!c || !path || (nfields > 0 && (!names || !arrays))) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        sysu::TecFields f;
        for (int k = 0; k < nfields; ++k) {
            std::string nm(names[k]);
            const double *a = arrays[k];
            if (nm == "P") f.P = a;
            else if (nm == "U") f.U = a;
            else if (nm == "V") f.V = a;
            else if (nm == "W") f.W = a;
            else if (nm == "R") f.R = a;
            else if (nm == "T") f.T = a;
            else if (nm == "VisLam") f.VisLam = a;
            else if (nm == "VisTur") f.VisTur = a;
            else if (nm == "TE") f.TE = a;
            else if (nm == "ED") f.ED = a;
            else if (nm == "solid_T") f.solid_T = a;
            else throw sysu::CaseError{"write_tecplot: unknown field " + nm};
        }
        sysu::write_tecplot(c->cs, path, f);
        return SYSU_OK;
    });
}

#define SYSU_METHOD(cname, call)                                                  \
    int cname(sysu_solver *s) {                                                   \
        if (!s) return set_err(SYSU_ERR_INPUT, "null argument");                  \
        return guarded([&] {                                                      \
            s->impl->call;                                                        \
            return SYSU_OK;                                                       \
        });                                                                       \
    }

SYSU_METHOD(sysu_solver_calculate_velocity, calculate_velocity())
SYSU_METHOD(sysu_solver_calculate_pressure, calculate_pressure())
SYSU_METHOD(sysu_solver_update_turkeps, update_ke())
SYSU_METHOD(sysu_solver_update_energy, update_energy())
SYSU_METHOD(sysu_solver_sync, sync())
SYSU_METHOD(sysu_solver_save_transient_old_data, save_transient_old_data())

int sysu_solver_heat_conduction(sysu_solver *s) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    if (!s->impl->cs.has_solid) return set_err(SYSU_ERR_INPUT, "case has no solid");
    return guarded([&] {
        s->impl->solid_solve();
        return SYSU_OK;
    });
}

int sysu_solver_check(sysu_solver *s) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        std::string msg = s->impl->check_iteration();
        if (!msg.empty()) return set_err(SYSU_ERR_SOLVE, msg);
        return SYSU_OK;
    });
}

int sysu_solver_reset(sysu_solver *s) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        s->impl->reset();
        return SYSU_OK;
    });
}

int sysu_solver_timer_start(sysu_solver *s) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        s->impl->timer_start();
        return SYSU_OK;
    });
}

int sysu_solver_timer_stop(sysu_solver *s, double *ms) {
    if (!s || !ms) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        *ms = s->impl->timer_stop();
        return SYSU_OK;
    });
}

long sysu_kernel_launches(void) { return sysu::g_launches.load(); }

int sysu_solver_spmv_timing(sysu_solver *s, const char *which, int fp32, int reps, double *ms) {
    if (!s || !which || !ms) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        *ms = s->impl->spmv_timing(which, fp32 != 0, reps, false);
        return SYSU_OK;
    });
}

int sysu_solver_spmv_timing_steady(sysu_solver *s, const char *which, int fp32, int reps, double *ms) {
    if (!s || !which || !ms) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        *ms = s->impl->spmv_timing(which, fp32 != 0, reps, true);
        return SYSU_OK;
    });
}

int sysu_solver_cg_phases(sysu_solver *s, unsigned long long *out, int n) {
    if (!s || !out) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        sysu::SimpleSolver &S = *s->impl;
        if (!S.phase_ts.get()) return set_err(SYSU_ERR_INPUT, "option profile_phases is off");
        int m = n < 256 ? n : 256;
        S.phase_ts.download(out, (size_t)m, S.st);
        S.sync();
        return SYSU_OK;
    });
}

int sysu_solver_residuals(sysu_solver *s, double *out10) {
    if (!s || !out10) return set_err(SYSU_ERR_INPUT, "null argument");
    for (int k = 0; k < 10; ++k) out10[k] = s->impl->Residual[k];
    return SYSU_OK;
}

int sysu_solver_solve_stats(sysu_solver *s, int *iters, double *res, int *status) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    for (int k = 0; k < sysu::SLOT_N; ++k)
        for (int c = 0; c < 3; ++c) {
            const sysu::SolveInfo &I = s->impl->last_info[k];
            if (iters) iters[k * 3 + c] = I.iters[c];
            if (res) res[k * 3 + c] = I.res[c];
            if (status) status[k * 3 + c] = I.status[c];
        }
    return SYSU_OK;
}

int sysu_solver_p_cycle(sysu_solver *s, const double *r, double *z, int use_net) {
    if (!s || !r || !z) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        s->impl->p_cycle(r, z, use_net != 0);
        return SYSU_OK;
    });
}

int sysu_solver_p_network(sysu_solver *s, int *level, float *params, int np) {
    if (!s || !level) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        sysu::SimpleSolver &S = *s->impl;
        const bool coarse = S.gnn.multigrid() == &S.mg && S.gnn.net_level >= 1;
        *level = coarse ? S.gnn.net_level : 0;
        sysu::GnnPrecond &g = coarse ? S.gnn_c : S.gnn;
        if (params) {
            if (np != sysu::GNN_NPARAM) throw sysu::CaseError{"sysu_solver_p_network: need sysu_gnn_num_params() values"};
            if (!g.bound()) throw sysu::CaseError{"sysu_solver_p_network: no network yet"};
            g.get_params(params, S.st);
        }
        return SYSU_OK;
    });
}

int sysu_solver_p_set_network(sysu_solver *s, const float *params, int np) {
    if (!s || !params || np != sysu::GNN_NPARAM) return set_err(SYSU_ERR_INPUT, "need sysu_gnn_num_params() values");
    return guarded([&] {
        sysu::SimpleSolver &S = *s->impl;
        const bool coarse = S.gnn.multigrid() == &S.mg && S.gnn.net_level >= 1;
        sysu::GnnPrecond &g = coarse ? S.gnn_c : S.gnn;
        if (!g.bound()) throw sysu::CaseError{"sysu_solver_p_set_network: no network yet"};
        g.set_params(params, S.st);
        return SYSU_OK;
    });
}

int sysu_solver_timing(sysu_solver *s, double *p_ms, double *mom_ms) {
    if (!s) return set_err(SYSU_ERR_INPUT, "null argument");
    if (p_ms) *p_ms = s->impl->last_p_ms;
    if (mom_ms) *mom_ms = s->impl->last_mom_ms;
    return SYSU_OK;
}

long sysu_solver_field_size(sysu_solver *s, const char *name) {
    if (!s || !name) return -1;
    return s->impl->field_size(name);
}

int sysu_solver_get_field(sysu_solver *s, const char *name, double *out, long n) {
    if (!s || !name || !out) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        s->impl->get_field(name, out, n);
        return SYSU_OK;
    });
}

int sysu_solver_set_field(sysu_solver *s, const char *name, const double *in, long n) {
    if (!s || !name || !in) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        s->impl->set_field(name, in, n);
        return SYSU_OK;
    });
}

// ---- batches of cases (batch.hpp) --------------------------------------------

struct sysu_batch {
    sysu::CaseBatch *impl;
};

int sysu_batch_create(int n, const char *const *params, sysu_batch **out) {
    if (!params || !out || n <= 0) return set_err(SYSU_ERR_INPUT, "sysu_batch_create: bad arguments");
    *out = nullptr;
    return guarded([&] {
        std::vector<std::string> ps;
        for (int k = 0; k < n; ++k) {
            if (!params[k]) throw sysu::CaseError{"sysu_batch_create: null param path"};
            ps.emplace_back(params[k]);
        }
        *out = new sysu_batch{new sysu::CaseBatch(ps)};
        return SYSU_OK;
    });
}

void sysu_batch_free(sysu_batch *b) {
    if (!b) return;
    try {
        delete b->impl;
    } catch (...) {
    }
    delete b;
}

void *sysu_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) {
        set_err(SYSU_ERR_CUDA, "cudaHostAlloc failed");
        return nullptr;
    }
    return p;
}

void sysu_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

int sysu_setup_phases(double *out) {
    if (!out) return set_err(SYSU_ERR_INPUT, "null argument");
    for (int k = 0; k < 5; ++k) out[k] = sysu::setup_phases()[k];
    return SYSU_OK;
}

int sysu_batch_size(sysu_batch *b) { return b ? b->impl->size() : 0; }

sysu_solver *sysu_batch_case(sysu_batch *b, int k) {
    if (!b || k < 0 || k >= b->impl->size()) return nullptr;
    return b->impl->handle(k);
}

int sysu_batch_tune(sysu_batch *b, const int *cand, int ncand, int *caps, double *ms_alone, double *ms_full,
                    double *makespan) {
    if (!b || !cand || ncand <= 0) return set_err(SYSU_ERR_INPUT, "sysu_batch_tune: bad arguments");
    return guarded([&] {
        sysu::TuneResult r = b->impl->tune(std::vector<int>(cand, cand + ncand));
        for (int k = 0; k < b->impl->size(); ++k) {
            if (caps) caps[k] = r.sm_cap[k];
            if (ms_alone) ms_alone[k] = r.ms_alone[k];
            if (ms_full) ms_full[k] = r.ms_full[k];
        }
        if (makespan) *makespan = r.measured_ms;
        return SYSU_OK;
    });
}

int sysu_batch_set_caps(sysu_batch *b, const int *caps) {
    if (!b || !caps) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        b->impl->set_caps(std::vector<int>(caps, caps + b->impl->size()));
        return SYSU_OK;
    });
}

int sysu_batch_capture(sysu_batch *b) {
    if (!b) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        b->impl->capture();
        return SYSU_OK;
    });
}

int sysu_batch_replay(sysu_batch *b, int n, double *ms) {
    if (!b || n < 0) return set_err(SYSU_ERR_INPUT, "bad arguments");
    return guarded([&] {
        double t = b->impl->replay(n);
        if (ms) *ms = t;
        return SYSU_OK;
    });
}

int sysu_batch_check(sysu_batch *b) {
    if (!b) return set_err(SYSU_ERR_INPUT, "null argument");
    return guarded([&] {
        std::string m = b->impl->check();
        if (!m.empty()) return set_err(SYSU_ERR_SOLVE, m);
        return SYSU_OK;
    });
}

int sysu_batch_run_sequential(sysu_batch *b, int n, double *ms) {
    if (!b || n < 0) return set_err(SYSU_ERR_INPUT, "bad arguments");
    return guarded([&] {
        double t = b->impl->run_sequential(n);
        if (ms) *ms = t;
        return SYSU_OK;
    });
}

}  // extern "C"
