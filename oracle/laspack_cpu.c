/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * CPU restatement of the LASPack API subset declared in laspack/laspack.h.
 * The reference links LASPack for every linear solve (tools.cpp:56-64); the
 * library itself is absent, so this file supplies the same entry points from
 * textbook algorithms (see the header for the sources).  Single-threaded and
 * deterministic, like the serial reference.
 *
 * Oracle-only switches, read from the environment at every iterator call, so
 * that the reference's hard-coded solver choices (navier_velocity.cpp:26,
 * navier_pressure.cpp:29, navier_scalar.cpp:101,143,374,
 * HeatConductionSolver.cpp:90) can be remapped without touching its source:
 *   SYSU_ORACLE_GMRES_AS   = GMRES | BiCGSTAB     (what GMRESIter runs)
 *   SYSU_ORACLE_CG_AS      = CG | BiCGSTAB        (what CGIter runs)
 *   SYSU_ORACLE_SSOR_AS    = SSOR | Jacobi | ILU  (what SSORPrecond applies)
 *   SYSU_ORACLE_RTC        = <eps>                (overrides SetRTCAccuracy)
 *   SYSU_ORACLE_MAXIT      = <n>     replaces every call site's iteration cap
 *                          (full-size parity runs at tight eps, where the
 *                          p' cap of 1000 would stop the solve first)
 *   SYSU_ORACLE_GMRES_M    = <restart length>     (default 10)
 *   SYSU_ORACLE_DUMP_DIR   = <dir>   dump A (full CSR), b, x0, x of each solve
 *   SYSU_ORACLE_DUMP_MAX   = <n>     number of solves to dump (default 16)
 */
#define _POSIX_C_SOURCE 199309L
#include "laspack/laspack.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------ */
/* global run-time-control state (LASPack keeps the same kind of globals)    */
static double g_rtc_eps = 1e-8;
static int g_last_iter = 0;
static double g_last_acc = 0.0;
static int g_gmres_m = 10;
static LaspackOracleStats g_stats;
static long g_solve_counter = 0;

const LaspackOracleStats *laspack_oracle_stats(void) { return &g_stats; }
void laspack_oracle_reset_stats(void) { memset(&g_stats, 0, sizeof g_stats); }

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void die(const char *msg) {
    fprintf(stderr, "laspack oracle: %s\n", msg);
    exit(3);
}

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) die("out of memory");
    return p;
}

static char *dupname(const char *s) {
    size_t n = s ? strlen(s) : 0;
    char *d = (char *)xmalloc(n + 1);
    if (n) memcpy(d, s, n);
    d[n] = '\0';
    return d;
}

/* ------------------------------------------------------------------------ */
/* vectors                                                                   */
void V_Constr(Vector *V, const char *Name, size_t Dim, InstanceType Instance, Boolean OwnData) {
    V->Name = dupname(Name);
    V->Dim = Dim;
    V->Instance = Instance;
    V->OwnData = OwnData;
    V->Cmp = (Real *)xmalloc((Dim + 1) * sizeof(Real));
    memset(V->Cmp, 0, (Dim + 1) * sizeof(Real));
}

void V_Destr(Vector *V) {
    free(V->Name);
    free(V->Cmp);
    V->Name = NULL;
    V->Cmp = NULL;
    V->Dim = 0;
}

void V_SetAllCmp(Vector *V, Real C) {
    for (size_t i = 1; i <= V->Dim; ++i) V->Cmp[i] = C;
}

/* ------------------------------------------------------------------------ */
/* matrices: row-wise storage as given by Q_SetLen / Q_SetEntry, plus a      */
/* cached full CSR view (0-based, both triangles) used by the iterators.     */
typedef struct {
    int valid;
    size_t n, nnz;
    size_t *rowptr;
    size_t *col;
    double *val;
    double *diag;
    /* ILU(0) factors share the CSR pattern (columns sorted per row) */
    int ilu_valid;
    double *ilu;
    size_t *diagpos;
} CsrView;

static CsrView *view_of(QMatrix *Q) {
    if (!Q->Priv) {
        Q->Priv = xmalloc(sizeof(CsrView));
        memset(Q->Priv, 0, sizeof(CsrView));
    }
    return (CsrView *)Q->Priv;
}

static void view_free(CsrView *v) {
    if (!v) return;
    free(v->rowptr);
    free(v->col);
    free(v->val);
    free(v->diag);
    free(v->ilu);
    free(v->diagpos);
    memset(v, 0, sizeof *v);
}

void Q_Constr(QMatrix *Q, const char *Name, size_t Dim, Boolean Symmetry,
              ElOrderType ElOrder, InstanceType Instance, Boolean OwnData) {
    Q->Name = dupname(Name);
    Q->Dim = Dim;
    Q->Symmetry = Symmetry;
    Q->ElOrder = ElOrder;
    Q->Instance = Instance;
    Q->OwnData = OwnData;
    Q->Len = (size_t *)xmalloc((Dim + 1) * sizeof(size_t));
    Q->El = (ElType **)xmalloc((Dim + 1) * sizeof(ElType *));
    for (size_t i = 0; i <= Dim; ++i) {
        Q->Len[i] = 0;
        Q->El[i] = NULL;
    }
    Q->Priv = NULL;
    if (ElOrder != Rowws) die("only row-wise matrices are supported");
}

void Q_Destr(QMatrix *Q) {
    if (Q->El)
        for (size_t i = 0; i <= Q->Dim; ++i) free(Q->El[i]);
    free(Q->El);
    free(Q->Len);
    free(Q->Name);
    if (Q->Priv) {
        view_free((CsrView *)Q->Priv);
        free(Q->Priv);
    }
    Q->El = NULL;
    Q->Len = NULL;
    Q->Name = NULL;
    Q->Priv = NULL;
}

void Q_SetLen(QMatrix *Q, size_t RoC, size_t Len) {
    if (RoC < 1 || RoC > Q->Dim) die("Q_SetLen: row out of range");
    free(Q->El[RoC]);
    Q->El[RoC] = (ElType *)xmalloc((Len ? Len : 1) * sizeof(ElType));
    for (size_t k = 0; k < Len; ++k) {
        Q->El[RoC][k].Pos = 0;
        Q->El[RoC][k].Val = 0.0;
    }
    Q->Len[RoC] = Len;
    if (Q->Priv) ((CsrView *)Q->Priv)->valid = 0;
}

void Q_SetEntry(QMatrix *Q, size_t RoC, size_t Entry, size_t Pos, Real Val) {
    if (RoC < 1 || RoC > Q->Dim || Entry >= Q->Len[RoC]) die("Q_SetEntry: index out of range");
    if (Pos < 1 || Pos > Q->Dim) die("Q_SetEntry: column out of range");
    if (Q->Symmetry && Pos < RoC) die("Q_SetEntry: symmetric matrix takes the upper triangle only");
    Q->El[RoC][Entry].Pos = Pos;
    Q->El[RoC][Entry].Val = Val;
    if (Q->Priv) ((CsrView *)Q->Priv)->valid = 0;
}

static int cmp_colval(const void *a, const void *b) {
    const size_t ca = *(const size_t *)a, cb = *(const size_t *)b;
    return (ca > cb) - (ca < cb);
}

/* Build the full CSR: per row the stored entries (then, for a symmetric
 * matrix, the mirrored entries of the lower triangle), sorted by column.
 * Duplicate columns in one row are summed. */
static CsrView *build_view(QMatrix *Q) {
    CsrView *v = view_of(Q);
    if (v->valid) return v;
    view_free(v);
    size_t n = Q->Dim;
    size_t *cnt = (size_t *)xmalloc((n + 1) * sizeof(size_t));
    for (size_t i = 0; i <= n; ++i) cnt[i] = 0;
    for (size_t r = 1; r <= n; ++r) {
        cnt[r - 1] += Q->Len[r];
        if (Q->Symmetry)
            for (size_t k = 0; k < Q->Len[r]; ++k)
                if (Q->El[r][k].Pos != r && Q->El[r][k].Pos != 0) cnt[Q->El[r][k].Pos - 1] += 1;
    }
    v->n = n;
    v->rowptr = (size_t *)xmalloc((n + 1) * sizeof(size_t));
    v->rowptr[0] = 0;
    for (size_t i = 0; i < n; ++i) v->rowptr[i + 1] = v->rowptr[i] + cnt[i];
    size_t cap = v->rowptr[n];
    /* (col,val) pairs for sorting */
    typedef struct { size_t c; double x; } CV;
    CV *tmp = (CV *)xmalloc(cap * sizeof(CV));
    size_t *fill = cnt;
    for (size_t i = 0; i < n; ++i) fill[i] = v->rowptr[i];
    for (size_t r = 1; r <= n; ++r) {
        for (size_t k = 0; k < Q->Len[r]; ++k) {
            size_t c = Q->El[r][k].Pos;
            if (c == 0) die("matrix row has an unset entry");
            tmp[fill[r - 1]].c = c - 1;
            tmp[fill[r - 1]].x = Q->El[r][k].Val;
            fill[r - 1]++;
            if (Q->Symmetry && c != r) {
                tmp[fill[c - 1]].c = r - 1;
                tmp[fill[c - 1]].x = Q->El[r][k].Val;
                fill[c - 1]++;
            }
        }
    }
    v->col = (size_t *)xmalloc(cap * sizeof(size_t));
    v->val = (double *)xmalloc(cap * sizeof(double));
    v->diag = (double *)xmalloc(n * sizeof(double));
    size_t out = 0;
    size_t *newptr = (size_t *)xmalloc((n + 1) * sizeof(size_t));
    newptr[0] = 0;
    for (size_t i = 0; i < n; ++i) {
        size_t b = v->rowptr[i], e = v->rowptr[i + 1];
        qsort(tmp + b, e - b, sizeof(CV), cmp_colval);
        v->diag[i] = 0.0;
        for (size_t k = b; k < e; ++k) {
            if (out > newptr[i] && v->col[out - 1] == tmp[k].c) {
                v->val[out - 1] += tmp[k].x;
            } else {
                v->col[out] = tmp[k].c;
                v->val[out] = tmp[k].x;
                out++;
            }
        }
        newptr[i + 1] = out;
        for (size_t k = newptr[i]; k < out; ++k)
            if (v->col[k] == i) v->diag[i] = v->val[k];
    }
    free(v->rowptr);
    v->rowptr = newptr;
    v->nnz = out;
    free(tmp);
    free(cnt);
    v->valid = 1;
    v->ilu_valid = 0;
    return v;
}

/* y = A x on 0-based arrays */
static void spmv(const CsrView *v, const double *x, double *y) {
    for (size_t i = 0; i < v->n; ++i) {
        double s = 0.0;
        for (size_t k = v->rowptr[i]; k < v->rowptr[i + 1]; ++k) s += v->val[k] * x[v->col[k]];
        y[i] = s;
    }
}

static double dot(const double *a, const double *b, size_t n) {
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* ------------------------------------------------------------------------ */
/* preconditioners: y = M^{-1} c                                             */
enum { PC_NONE, PC_JACOBI, PC_SSOR, PC_ILU };

static void pc_jacobi(const CsrView *v, double *y, const double *c, double omega) {
    for (size_t i = 0; i < v->n; ++i) {
        if (v->diag[i] == 0.0) die("Jacobi: zero diagonal");
        y[i] = omega * c[i] / v->diag[i];
    }
}

/* SSOR: M = (D/w + L) (w/(2-w)) (D/w)^{-1} ... written as
 * y = w(2-w) (D + wU)^{-1} D (D + wL)^{-1} c   (Saad, sect. 10.2.1) */
static void pc_ssor(const CsrView *v, double *y, const double *c, double omega) {
    size_t n = v->n;
    for (size_t i = 0; i < n; ++i) {
        double s = c[i];
        for (size_t k = v->rowptr[i]; k < v->rowptr[i + 1]; ++k)
            if (v->col[k] < i) s -= omega * v->val[k] * y[v->col[k]];
        if (v->diag[i] == 0.0) die("SSOR: zero diagonal");
        y[i] = s / v->diag[i];
    }
    for (size_t i = 0; i < n; ++i) y[i] *= v->diag[i];
    for (size_t ii = n; ii-- > 0;) {
        double s = y[ii];
        for (size_t k = v->rowptr[ii]; k < v->rowptr[ii + 1]; ++k)
            if (v->col[k] > ii) s -= omega * v->val[k] * y[v->col[k]];
        y[ii] = s / v->diag[ii];
    }
    double f = omega * (2.0 - omega);
    for (size_t i = 0; i < n; ++i) y[i] *= f;
}

/* ILU(0), IKJ variant (Saad Alg. 10.4) on the full CSR pattern. */
static void ilu_factor(CsrView *v) {
    if (v->ilu_valid) return;
    size_t n = v->n;
    free(v->ilu);
    free(v->diagpos);
    v->ilu = (double *)xmalloc(v->nnz * sizeof(double));
    v->diagpos = (size_t *)xmalloc(n * sizeof(size_t));
    memcpy(v->ilu, v->val, v->nnz * sizeof(double));
    long *pos = (long *)xmalloc(n * sizeof(long));
    for (size_t i = 0; i < n; ++i) pos[i] = -1;
    for (size_t i = 0; i < n; ++i) {
        v->diagpos[i] = (size_t)-1;
        for (size_t k = v->rowptr[i]; k < v->rowptr[i + 1]; ++k) {
            pos[v->col[k]] = (long)k;
            if (v->col[k] == i) v->diagpos[i] = k;
        }
        if (v->diagpos[i] == (size_t)-1) die("ILU: missing diagonal");
        for (size_t k = v->rowptr[i]; k < v->rowptr[i + 1]; ++k) {
            size_t j = v->col[k];
            if (j >= i) break;
            double lij = v->ilu[k] / v->ilu[v->diagpos[j]];
            v->ilu[k] = lij;
            for (size_t kk = v->diagpos[j] + 1; kk < v->rowptr[j + 1]; ++kk) {
                long p = pos[v->col[kk]];
                if (p >= 0) v->ilu[p] -= lij * v->ilu[kk];
            }
        }
        if (v->ilu[v->diagpos[i]] == 0.0) die("ILU: zero pivot");
        for (size_t k = v->rowptr[i]; k < v->rowptr[i + 1]; ++k) pos[v->col[k]] = -1;
    }
    free(pos);
    v->ilu_valid = 1;
}

static void pc_ilu(CsrView *v, double *y, const double *c) {
    ilu_factor(v);
    size_t n = v->n;
    for (size_t i = 0; i < n; ++i) {
        double s = c[i];
        for (size_t k = v->rowptr[i]; k < v->diagpos[i]; ++k) s -= v->ilu[k] * y[v->col[k]];
        y[i] = s;
    }
    for (size_t ii = n; ii-- > 0;) {
        double s = y[ii];
        for (size_t k = v->diagpos[ii] + 1; k < v->rowptr[ii + 1]; ++k) s -= v->ilu[k] * y[v->col[k]];
        y[ii] = s / v->ilu[v->diagpos[ii]];
    }
}

static const char *env_or(const char *k, const char *def) {
    const char *s = getenv(k);
    return (s && *s) ? s : def;
}

static int remap_precond(int pc) {
    if (pc != PC_SSOR) return pc;
    const char *s = env_or("SYSU_ORACLE_SSOR_AS", "SSOR");
    if (strcmp(s, "Jacobi") == 0) return PC_JACOBI;
    if (strcmp(s, "ILU") == 0) return PC_ILU;
    return PC_SSOR;
}

static void apply_pc(int pc, CsrView *v, double *y, const double *c, double omega) {
    switch (pc) {
    case PC_NONE: memcpy(y, c, v->n * sizeof(double)); break;
    case PC_JACOBI: pc_jacobi(v, y, c, omega); break;
    case PC_SSOR: pc_ssor(v, y, c, omega); break;
    case PC_ILU: pc_ilu(v, y, c); break;
    }
}

/* The public preconditioner entry points (LASPack convention: y = M^-1 c,
 * vectors 1-based).  Iterators recognise them by address and call the
 * 0-based kernels directly. */
Vector *JacobiPrecond(QMatrix *A, Vector *y, Vector *c, double Omega) {
    CsrView *v = build_view(A);
    pc_jacobi(v, y->Cmp + 1, c->Cmp + 1, Omega);
    return y;
}
Vector *SSORPrecond(QMatrix *A, Vector *y, Vector *c, double Omega) {
    CsrView *v = build_view(A);
    apply_pc(remap_precond(PC_SSOR), v, y->Cmp + 1, c->Cmp + 1, Omega);
    return y;
}
Vector *ILUPrecond(QMatrix *A, Vector *y, Vector *c, double Omega) {
    (void)Omega;
    CsrView *v = build_view(A);
    pc_ilu(v, y->Cmp + 1, c->Cmp + 1);
    return y;
}

static int pc_kind(PrecondProcType p) {
    if (p == NULL) return PC_NONE;
    if (p == JacobiPrecond) return PC_JACOBI;
    if (p == SSORPrecond) return remap_precond(PC_SSOR);
    if (p == ILUPrecond) return PC_ILU;
    die("unknown preconditioner procedure");
    return PC_NONE;
}

/* ------------------------------------------------------------------------ */
void SetRTCAccuracy(double NewEps) { g_rtc_eps = NewEps; }
int GetLastNoIter(void) { return g_last_iter; }
double GetLastAccuracy(void) { return g_last_acc; }
void SetGMRESRestart(int MaxSteps) { g_gmres_m = MaxSteps > 0 ? MaxSteps : 10; }

static double effective_eps(void) {
    const char *s = getenv("SYSU_ORACLE_RTC");
    if (s && *s) return atof(s);
    return g_rtc_eps;
}

/* Krylov kernels on 0-based arrays.  Each returns the iteration count and
 * stores the final relative residual in *acc. */
static int cg_run(CsrView *v, double *x, const double *b, int maxit, int pc, double omega,
                  double eps, double *acc) {
    size_t n = v->n;
    double *r = (double *)xmalloc(n * sizeof(double));
    double *z = (double *)xmalloc(n * sizeof(double));
    double *p = (double *)xmalloc(n * sizeof(double));
    double *q = (double *)xmalloc(n * sizeof(double));
    double bnorm = sqrt(dot(b, b, n));
    if (bnorm == 0.0) bnorm = 1.0;
    spmv(v, x, q);
    for (size_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
    double res = sqrt(dot(r, r, n)) / bnorm;
    int it = 0;
    double rho_prev = 1.0;
    while (!(res < eps) && it < maxit) {
        ++it;
        apply_pc(pc, v, z, r, omega);
        double rho = dot(r, z, n);
        if (it == 1) {
            memcpy(p, z, n * sizeof(double));
        } else {
            double beta = rho / rho_prev;
            for (size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        }
        spmv(v, p, q);
        double pq = dot(p, q, n);
        if (pq == 0.0) break;
        double alpha = rho / pq;
        for (size_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        res = sqrt(dot(r, r, n)) / bnorm;
        rho_prev = rho;
    }
    free(r); free(z); free(p); free(q);
    *acc = res;
    return it;
}

static int bicgstab_run(CsrView *v, double *x, const double *b, int maxit, int pc, double omega_pc,
                        double eps, double *acc) {
    size_t n = v->n;
    double *r = (double *)xmalloc(n * sizeof(double));
    double *rt = (double *)xmalloc(n * sizeof(double));
    double *p = (double *)xmalloc(n * sizeof(double));
    double *ph = (double *)xmalloc(n * sizeof(double));
    double *vv = (double *)xmalloc(n * sizeof(double));
    double *s = (double *)xmalloc(n * sizeof(double));
    double *sh = (double *)xmalloc(n * sizeof(double));
    double *t = (double *)xmalloc(n * sizeof(double));
    double bnorm = sqrt(dot(b, b, n));
    if (bnorm == 0.0) bnorm = 1.0;
    spmv(v, x, t);
    for (size_t i = 0; i < n; ++i) r[i] = b[i] - t[i];
    memcpy(rt, r, n * sizeof(double));
    double res = sqrt(dot(r, r, n)) / bnorm;
    int it = 0;
    double rho_prev = 1.0, alpha = 1.0, omega = 1.0;
    while (!(res < eps) && it < maxit) {
        double rho = dot(rt, r, n);
        if (rho == 0.0) break;
        ++it;
        if (it == 1) {
            memcpy(p, r, n * sizeof(double));
        } else {
            double beta = (rho / rho_prev) * (alpha / omega);
            for (size_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * vv[i]);
        }
        apply_pc(pc, v, ph, p, omega_pc);
        spmv(v, ph, vv);
        double rtv = dot(rt, vv, n);
        if (rtv == 0.0) break;
        alpha = rho / rtv;
        for (size_t i = 0; i < n; ++i) s[i] = r[i] - alpha * vv[i];
        double snorm = sqrt(dot(s, s, n)) / bnorm;
        if (snorm < eps) {
            for (size_t i = 0; i < n; ++i) x[i] += alpha * ph[i];
            res = snorm;
            break;
        }
        apply_pc(pc, v, sh, s, omega_pc);
        spmv(v, sh, t);
        double tt = dot(t, t, n);
        omega = tt != 0.0 ? dot(t, s, n) / tt : 0.0;
        for (size_t i = 0; i < n; ++i) {
            x[i] += alpha * ph[i] + omega * sh[i];
            r[i] = s[i] - omega * t[i];
        }
        res = sqrt(dot(r, r, n)) / bnorm;
        rho_prev = rho;
        if (omega == 0.0) break;
    }
    free(r); free(rt); free(p); free(ph); free(vv); free(s); free(sh); free(t);
    *acc = res;
    return it;
}

/* Restarted GMRES(m), right preconditioned, modified Gram-Schmidt and
 * Givens rotations (Saad Alg. 9.5). */
static int gmres_run(CsrView *v, double *x, const double *b, int maxit, int pc, double omega_pc,
                     double eps, double *acc) {
    size_t n = v->n;
    const char *ms = getenv("SYSU_ORACLE_GMRES_M");
    int m = (ms && *ms) ? atoi(ms) : g_gmres_m;
    if (m < 1) m = 10;
    double *V = (double *)xmalloc((size_t)(m + 1) * n * sizeof(double));
    double *Z = (double *)xmalloc((size_t)m * n * sizeof(double));
    double *H = (double *)xmalloc((size_t)(m + 1) * m * sizeof(double));
    double *cs = (double *)xmalloc(m * sizeof(double));
    double *sn = (double *)xmalloc(m * sizeof(double));
    double *g = (double *)xmalloc((m + 1) * sizeof(double));
    double *yv = (double *)xmalloc(m * sizeof(double));
    double *w = (double *)xmalloc(n * sizeof(double));
    double bnorm = sqrt(dot(b, b, n));
    if (bnorm == 0.0) bnorm = 1.0;
    int it = 0;
    double res;
    for (;;) {
        spmv(v, x, w);
        for (size_t i = 0; i < n; ++i) V[i] = b[i] - w[i];
        double beta = sqrt(dot(V, V, n));
        res = beta / bnorm;
        if (res < eps || it >= maxit || beta == 0.0) break;
        for (size_t i = 0; i < n; ++i) V[i] /= beta;
        for (int k = 0; k <= m; ++k) g[k] = 0.0;
        g[0] = beta;
        int j = 0;
        for (; j < m && it < maxit; ++j) {
            ++it;
            double *zj = Z + (size_t)j * n;
            apply_pc(pc, v, zj, V + (size_t)j * n, omega_pc);
            spmv(v, zj, w);
            for (int k = 0; k <= j; ++k) {
                double *vk = V + (size_t)k * n;
                double h = dot(w, vk, n);
                H[k * m + j] = h;
                for (size_t i = 0; i < n; ++i) w[i] -= h * vk[i];
            }
            double hn = sqrt(dot(w, w, n));
            H[(j + 1) * m + j] = hn;
            if (hn != 0.0) {
                double *vn = V + (size_t)(j + 1) * n;
                for (size_t i = 0; i < n; ++i) vn[i] = w[i] / hn;
            }
            for (int k = 0; k < j; ++k) {
                double a = H[k * m + j], c2 = H[(k + 1) * m + j];
                H[k * m + j] = cs[k] * a + sn[k] * c2;
                H[(k + 1) * m + j] = -sn[k] * a + cs[k] * c2;
            }
            double a = H[j * m + j], c2 = H[(j + 1) * m + j];
            double den = sqrt(a * a + c2 * c2);
            cs[j] = den != 0.0 ? a / den : 1.0;
            sn[j] = den != 0.0 ? c2 / den : 0.0;
            H[j * m + j] = den;
            H[(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            res = fabs(g[j + 1]) / bnorm;
            if (res < eps || hn == 0.0) { ++j; break; }
        }
        for (int k = j - 1; k >= 0; --k) {
            double s = g[k];
            for (int l = k + 1; l < j; ++l) s -= H[k * m + l] * yv[l];
            yv[k] = s / H[k * m + k];
        }
        for (int k = 0; k < j; ++k) {
            double *zk = Z + (size_t)k * n;
            for (size_t i = 0; i < n; ++i) x[i] += yv[k] * zk[i];
        }
        if (res < eps || it >= maxit) {
            spmv(v, x, w);
            double s2 = 0.0;
            for (size_t i = 0; i < n; ++i) { double d = b[i] - w[i]; s2 += d * d; }
            res = sqrt(s2) / bnorm;
            if (res < eps || it >= maxit) break;
        }
    }
    free(V); free(Z); free(H); free(cs); free(sn); free(g); free(yv); free(w);
    *acc = res;
    return it;
}

/* ------------------------------------------------------------------------ */
static void dump_array(const char *dir, long k, const char *tag, const void *p, size_t bytes) {
    char path[1024];
    snprintf(path, sizeof path, "%s/solve_%04ld_%s", dir, k, tag);
    FILE *f = fopen(path, "wb");
    if (!f) return;
    fwrite(p, 1, bytes, f);
    fclose(f);
}

enum { M_CG = 0, M_BICGSTAB = 1, M_GMRES = 2 };
static const char *mname[3] = {"CG", "BiCGSTAB", "GMRES"};
static const char *pname[4] = {"none", "Jacobi", "SSOR", "ILU"};

static Vector *run_iter(int method, QMatrix *A, Vector *x, Vector *b, int MaxIter,
                        PrecondProcType Precond, double Omega) {
    if (method == M_GMRES && strcmp(env_or("SYSU_ORACLE_GMRES_AS", "GMRES"), "BiCGSTAB") == 0)
        method = M_BICGSTAB;
    if (method == M_CG && strcmp(env_or("SYSU_ORACLE_CG_AS", "CG"), "BiCGSTAB") == 0)
        method = M_BICGSTAB;
    int pc = pc_kind(Precond);
    double eps = effective_eps();
    const char *mi = getenv("SYSU_ORACLE_MAXIT");
    if (mi && *mi && atoi(mi) > 0) MaxIter = atoi(mi);
    CsrView *v = build_view(A);
    size_t n = v->n;
    if (x->Dim != n || b->Dim != n) die("dimension mismatch");
    long k = g_solve_counter++;
    const char *dd = getenv("SYSU_ORACLE_DUMP_DIR");
    long dmax = atol(env_or("SYSU_ORACLE_DUMP_MAX", "16"));
    int dumping = dd && *dd && k < dmax;
    if (dumping) {
        int *rp = (int *)xmalloc((n + 1) * sizeof(int));
        int *cl = (int *)xmalloc(v->nnz * sizeof(int));
        for (size_t i = 0; i <= n; ++i) rp[i] = (int)v->rowptr[i];
        for (size_t i = 0; i < v->nnz; ++i) cl[i] = (int)v->col[i];
        dump_array(dd, k, "rowptr.i32", rp, (n + 1) * sizeof(int));
        dump_array(dd, k, "col.i32", cl, v->nnz * sizeof(int));
        dump_array(dd, k, "val.f64", v->val, v->nnz * sizeof(double));
        dump_array(dd, k, "b.f64", b->Cmp + 1, n * sizeof(double));
        dump_array(dd, k, "x0.f64", x->Cmp + 1, n * sizeof(double));
        free(rp);
        free(cl);
    }
    double t0 = now_s();
    double acc = 0.0;
    int it = 0;
    switch (method) {
    case M_CG: it = cg_run(v, x->Cmp + 1, b->Cmp + 1, MaxIter, pc, Omega, eps, &acc); break;
    case M_BICGSTAB: it = bicgstab_run(v, x->Cmp + 1, b->Cmp + 1, MaxIter, pc, Omega, eps, &acc); break;
    default: it = gmres_run(v, x->Cmp + 1, b->Cmp + 1, MaxIter, pc, Omega, eps, &acc); break;
    }
    double t1 = now_s();
    g_stats.calls[method] += 1;
    g_stats.iters[method] += it;
    g_stats.seconds[method] += t1 - t0;
    g_last_iter = it;
    g_last_acc = acc;
    if (dumping) {
        dump_array(dd, k, "x.f64", x->Cmp + 1, n * sizeof(double));
        char path[1024];
        snprintf(path, sizeof path, "%s/solves.txt", dd);
        FILE *f = fopen(path, "a");
        if (f) {
            fprintf(f, "%ld %s %s %zu %zu %.17g %d %.17g %d %.17g %d\n", k, mname[method], pname[pc], n,
                    v->nnz, eps, MaxIter, Omega, it, acc, (int)A->Symmetry);
            fclose(f);
        }
    }
    return x;
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
