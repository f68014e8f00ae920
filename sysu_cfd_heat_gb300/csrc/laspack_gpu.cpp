// LASPack-compatible C ABI on the GPU (declared in include/laspack/laspack.h).
//
// Matrices are assembled on the host exactly as LASPack stores them (rows of
// (column, value) pairs, upper triangle only for symmetric matrices); at each
// iterator call the rows are flattened into a full CSR with the diagonal
// first, converted to SELL-32 and solved by the persistent Krylov kernels.
// The SELL pattern is cached by content, so the reference's habit of
// constructing and destroying the same matrix every outer iteration
// (navier_velocity.cpp:19,73) costs one value upload per solve, not a new
// pattern.
#include "../../include/laspack/laspack.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <vector>

#include "krylov.hpp"

namespace {

using namespace sysu;

struct Pattern {
    int n = 0;
    std::vector<int> rowptr, cols;  // full CSR, diagonal first
    uint64_t hash = 0;
};

struct DevMatrix {
    Pattern key;
    SellPattern pat;
    SellDev A;
    DevBuf<double> val, x, b, y;
    std::vector<double> hval;
};

struct State {
    std::mutex mu;
    double eps = 1e-8;
    int last_iter = 0;
    double last_acc = 0.0;
    int gmres_as = 0, ssor_as = 0;  // laspack_gpu_set_mode: 0 = the named method
    int restart = 10;               // SetGMRESRestart
    long solves = 0, iters = 0;
    bool warned_gmres = false, warned_ssor = false, warned_err = false;
    cudaStream_t st = nullptr;
    KrylovWork work;
    DevBuf<SolveInfo> info;
    std::list<std::unique_ptr<DevMatrix>> cache;  // most recently used first
};

State &S() {
    static State s;
    return s;
}

char *dupname(const char *s) {
    size_t n = s ? std::strlen(s) : 0;
    char *d = (char *)std::malloc(n + 1);
    if (n) std::memcpy(d, s, n);
    d[n] = '\0';
    return d;
}

void flatten(const QMatrix *Q, Pattern &p, std::vector<double> &vals) {
    size_t n = Q->Dim;
    p.n = (int)n;
    std::vector<std::vector<std::pair<int, double>>> lower;
    if (Q->Symmetry) lower.resize(n);
    if (Q->Symmetry)
        for (size_t r = 1; r <= n; ++r)
            for (size_t k = 0; k < Q->Len[r]; ++k) {
                size_t c = Q->El[r][k].Pos;
                if (c != r && c >= 1 && c <= n) lower[c - 1].push_back({(int)(r - 1), Q->El[r][k].Val});
            }
    p.rowptr.assign(n + 1, 0);
    p.cols.clear();
    vals.clear();
    uint64_t h = 1469598103934665603ull;
    for (size_t r = 1; r <= n; ++r) {
        double d = 0.0;
        for (size_t k = 0; k < Q->Len[r]; ++k)
            if (Q->El[r][k].Pos == r) d += Q->El[r][k].Val;
        p.cols.push_back((int)(r - 1));
        vals.push_back(d);
        for (size_t k = 0; k < Q->Len[r]; ++k) {
            size_t c = Q->El[r][k].Pos;
            if (c == r) continue;
            if (c < 1 || c > n) throw CaseError{"matrix entry with a column out of range"};
            p.cols.push_back((int)(c - 1));
            vals.push_back(Q->El[r][k].Val);
        }
        if (Q->Symmetry)
            for (auto &e : lower[r - 1]) {
                p.cols.push_back(e.first);
                vals.push_back(e.second);
            }
        p.rowptr[r] = (int)p.cols.size();
    }
    for (int c : p.cols) h = (h ^ (uint64_t)(uint32_t)c) * 1099511628211ull;
    for (int r : p.rowptr) h = (h ^ (uint64_t)(uint32_t)r) * 1099511628211ull;
    p.hash = h;
}

DevMatrix &matrix_for(State &s, const Pattern &p) {
    for (auto it = s.cache.begin(); it != s.cache.end(); ++it) {
        DevMatrix &m = **it;
        if (m.key.hash == p.hash && m.key.n == p.n && m.key.rowptr == p.rowptr && m.key.cols == p.cols) {
            s.cache.splice(s.cache.begin(), s.cache, it);
            return *s.cache.front();
        }
    }
    auto m = std::make_unique<DevMatrix>();
    m->key = p;
    m->pat = make_sell(p.n, p.rowptr, p.cols);
    m->A.upload(m->pat, s.st);
    m->val.alloc(m->pat.nnz);
    m->val.zero(s.st);
    m->hval.assign(m->pat.nnz, 0.0);
    m->x.alloc(p.n);
    m->b.alloc(p.n);
    m->y.alloc(p.n);
    s.cache.push_front(std::move(m));
    while (s.cache.size() > 6) s.cache.pop_back();
    return *s.cache.front();
}

enum { M_CG = 0, M_BICGSTAB = 1, M_GMRES = 2 };

// The preconditioner a LASPack iterator was given, by address: these three
// (and none) run on the GPU; any other function is refused (no CPU fallback).
int precond_kind(PrecondProcType pc) {
    if (pc == nullptr) return PK_NONE;
    if (pc == JacobiPrecond) return PK_JACOBI;
    if (pc == SSORPrecond) return PK_SSOR;
    if (pc == ILUPrecond) return PK_ILU0;
    throw CaseError{"unknown preconditioner function: only JacobiPrecond, SSORPrecond, ILUPrecond run on the GPU"};
}

Vector *run_iter(int method, QMatrix *A, Vector *x, Vector *b, int MaxIter, PrecondProcType pc, double Omega) {
    State &s = S();
    std::lock_guard<std::mutex> lock(s.mu);
    try {
        if (!s.st) {
            SYSU_CUDA(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
            s.info.alloc(1);
        }
        if (x->Dim != A->Dim || b->Dim != A->Dim) throw CaseError{"dimension mismatch"};
        Pattern p;
        std::vector<double> vals;
        flatten(A, p, vals);
        DevMatrix &m = matrix_for(s, p);
        for (int i = 0; i < p.n; ++i)
            for (int k = p.rowptr[i]; k < p.rowptr[i + 1]; ++k) m.hval[m.pat.pos(i, k - p.rowptr[i])] = vals[k];
        m.val.upload(m.hval.data(), m.hval.size(), s.st);
        m.b.upload(b->Cmp + 1, p.n, s.st);
        m.x.upload(x->Cmp + 1, p.n, s.st);
        KrylovOpts o;
        o.maxit = MaxIter;
        o.eps = s.eps;
        if (const char *ov = std::getenv("SYSU_LASPACK_RTC")) o.eps = std::atof(ov);
        o.omega = Omega;
        int kind = precond_kind(pc);
        if ((kind == PK_SSOR || kind == PK_ILU0) && s.ssor_as == 1) {
            if (!s.warned_ssor) {
                std::fprintf(stderr, "laspack (GPU): SSOR/ILU preconditioners run as Jacobi (laspack_gpu_set_mode)\n");
                s.warned_ssor = true;
            }
            kind = PK_JACOBI;
        }
        if (method == M_GMRES && s.gmres_as == 1) {
            if (!s.warned_gmres) {
                std::fprintf(stderr, "laspack (GPU): GMRESIter runs BiCGSTAB (laspack_gpu_set_mode)\n");
                s.warned_gmres = true;
            }
            method = M_BICGSTAB;
        }
        if (method == M_BICGSTAB && (kind == PK_SSOR || kind == PK_ILU0)) {
            if (!s.warned_ssor) {
                std::fprintf(stderr, "laspack (GPU): BiCGSTABIter applies the Jacobi preconditioner\n");
                s.warned_ssor = true;
            }
            kind = PK_JACOBI;
        }
        o.jacobi = kind == PK_JACOBI;
        if (method == M_CG) {
            if (kind == PK_JACOBI || kind == PK_NONE)
                cg_solve(m.A, m.val.get(), m.b.get(), m.x.get(), false, o, s.work, s.info.get(), s.st);
            else
                pcg_solve(m.A, m.val.get(), m.b.get(), m.x.get(), false, o, kind, s.work, s.info.get(), s.st);
        } else if (method == M_GMRES) {
            gmres_solve(m.A, m.val.get(), m.b.get(), m.x.get(), false, o, kind, s.restart, s.work, s.info.get(), s.st);
        } else {
            const double *bb[1] = {m.b.get()};
            double *xx[1] = {m.x.get()};
            bicgstab_solve(m.A, m.val.get(), 1, bb, xx, o, s.work, s.info.get(), s.st);
        }
        SolveInfo h;
        s.info.download(&h, 1, s.st);
        m.x.download(x->Cmp + 1, p.n, s.st);
        SYSU_CUDA(cudaStreamSynchronize(s.st));
        if (h.err) throw CaseError{"Krylov solve aborted: a grid barrier wait timed out"};
        s.last_iter = h.iters[0];
        s.last_acc = h.res[0];
        s.solves += 1;
        s.iters += h.iters[0];
    } catch (const CaseError &e) {
        if (!s.warned_err) {
            std::fprintf(stderr, "laspack (GPU): solve failed: %s\n", e.msg.c_str());
            s.warned_err = true;
        }
        // make the caller's own convergence checks fire (navier_velocity.cpp:29,
        // navier_pressure.cpp:32): no silent success without a GPU
        s.last_iter = MaxIter;
        s.last_acc = INFINITY;
    }
    return x;
}

Vector *precond_apply(int kind, QMatrix *A, Vector *y, Vector *c, double Omega) {
    State &s = S();
    std::lock_guard<std::mutex> lock(s.mu);
    try {
        if (!s.st) {
            SYSU_CUDA(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
            s.info.alloc(1);
        }
        Pattern p;
        std::vector<double> vals;
        flatten(A, p, vals);
        DevMatrix &m = matrix_for(s, p);
        for (int i = 0; i < p.n; ++i)
            for (int k = p.rowptr[i]; k < p.rowptr[i + 1]; ++k) m.hval[m.pat.pos(i, k - p.rowptr[i])] = vals[k];
        m.val.upload(m.hval.data(), m.hval.size(), s.st);
        m.b.upload(c->Cmp + 1, p.n, s.st);
        if ((kind == PK_SSOR || kind == PK_ILU0) && s.ssor_as == 1) kind = PK_JACOBI;
        precond_solve(m.A, m.val.get(), kind, Omega, m.b.get(), m.y.get(), s.work, s.info.get(), s.st);
        SolveInfo h;
        s.info.download(&h, 1, s.st);
        m.y.download(y->Cmp + 1, p.n, s.st);
        SYSU_CUDA(cudaStreamSynchronize(s.st));
        if (h.err) throw CaseError{"preconditioner aborted: a grid barrier wait timed out"};
        if (h.status[1]) throw CaseError{"ILU(0): zero pivot or row longer than 16 entries"};
    } catch (const CaseError &e) {
        std::fprintf(stderr, "laspack (GPU): preconditioner failed: %s\n", e.msg.c_str());
        for (size_t i = 1; i <= y->Dim; ++i) y->Cmp[i] = NAN;
    }
    return y;
}

}  // namespace

extern "C" {

void Q_Constr(QMatrix *Q, const char *Name, size_t Dim, Boolean Symmetry, ElOrderType ElOrder,
              InstanceType Instance, Boolean OwnData) {
    Q->Name = dupname(Name);
    Q->Dim = Dim;
    Q->Symmetry = Symmetry;
    Q->ElOrder = ElOrder;
    Q->Instance = Instance;
    Q->OwnData = OwnData;
    Q->Len = (size_t *)std::calloc(Dim + 1, sizeof(size_t));
    Q->El = (ElType **)std::calloc(Dim + 1, sizeof(ElType *));
    Q->Priv = nullptr;
}

void Q_Destr(QMatrix *Q) {
    if (Q->El)
        for (size_t i = 0; i <= Q->Dim; ++i) std::free(Q->El[i]);
    std::free(Q->El);
    std::free(Q->Len);
    std::free(Q->Name);
    Q->El = nullptr;
    Q->Len = nullptr;
    Q->Name = nullptr;
}

void Q_SetLen(QMatrix *Q, size_t RoC, size_t Len) {
    if (RoC < 1 || RoC > Q->Dim) return;
    std::free(Q->El[RoC]);
    Q->El[RoC] = (ElType *)std::calloc(Len ? Len : 1, sizeof(ElType));
    Q->Len[RoC] = Len;
}

void Q_SetEntry(QMatrix *Q, size_t RoC, size_t Entry, size_t Pos, Real Val) {
    if (RoC < 1 || RoC > Q->Dim || Entry >= Q->Len[RoC]) return;
    Q->El[RoC][Entry].Pos = Pos;
    Q->El[RoC][Entry].Val = Val;
}

void V_Constr(Vector *V, const char *Name, size_t Dim, InstanceType Instance, Boolean OwnData) {
    V->Name = dupname(Name);
    V->Dim = Dim;
    V->Instance = Instance;
    V->OwnData = OwnData;
    V->Cmp = (Real *)std::calloc(Dim + 1, sizeof(Real));
}

void V_Destr(Vector *V) {
    std::free(V->Name);
    std::free(V->Cmp);
    V->Name = nullptr;
    V->Cmp = nullptr;
    V->Dim = 0;
}

void V_SetAllCmp(Vector *V, Real C) {
    for (size_t i = 1; i <= V->Dim; ++i) V->Cmp[i] = C;
}

void SetRTCAccuracy(double NewEps) { S().eps = NewEps; }
int GetLastNoIter(void) { return S().last_iter; }
double GetLastAccuracy(void) { return S().last_acc; }
void SetGMRESRestart(int MaxSteps) {
    State &s = S();
    s.restart = MaxSteps < 1 ? 10 : (MaxSteps > GMRES_MAX_RESTART ? GMRES_MAX_RESTART : MaxSteps);
}

Vector *CGIter(QMatrix *A, Vector *x, Vector *b, int MaxIter, PrecondProcType Precond, double Omega) {
    return run_iter(M_CG, A, x, b, MaxIter, Precond, Omega);
}
Vector *BiCGSTABIter(QMatrix *A, Vector *x, Vector *b, int MaxIter, PrecondProcType Precond, double Omega) {
    return run_iter(M_BICGSTAB, A, x, b, MaxIter, Precond, Omega);
}
Vector *GMRESIter(QMatrix *A, Vector *x, Vector *b, int MaxIter, PrecondProcType Precond, double Omega) {
    return run_iter(M_GMRES, A, x, b, MaxIter, Precond, Omega);
}

Vector *JacobiPrecond(QMatrix *A, Vector *y, Vector *c, double Omega) {
    return precond_apply(PK_JACOBI, A, y, c, Omega);
}
Vector *SSORPrecond(QMatrix *A, Vector *y, Vector *c, double Omega) { return precond_apply(PK_SSOR, A, y, c, Omega); }
Vector *ILUPrecond(QMatrix *A, Vector *y, Vector *c, double Omega) { return precond_apply(PK_ILU0, A, y, c, Omega); }

int laspack_gpu_set_mode(int gmres_as, int ssor_as) {
    S().gmres_as = gmres_as;
    S().ssor_as = ssor_as;
    return 0;
}
long laspack_gpu_solves(void) { return S().solves; }
long laspack_gpu_iterations(void) { return S().iters; }

}  // extern "C"
