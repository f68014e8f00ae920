// General-preconditioner Krylov solvers: restarted GMRES(m) and PCG with the
// preconditioners LASPack offers the reference (JacobiPrecond, SSORPrecond,
// ILUPrecond), as persistent cooperative kernels (FP64).
//
// These are the reference's default solver mode: momentum and scalars through
// GMRESIter + SSORPrecond (navier_velocity.cpp:26, navier_scalar.cpp:101,143,374),
// p' and solid conduction through CGIter + SSORPrecond (navier_pressure.cpp:29,
// HeatConductionSolver.cpp:90).  The algorithms follow the oracle's LASPack
// restatement:
//   SSOR(w):  y = w(2-w) (D + wU)^-1 D (D + wL)^-1 c          (Saad 10.2.1)
//   ILU(0):   IKJ factorisation on the matrix pattern            (Saad Alg. 10.4)
//   GMRES(m): right preconditioned, Givens rotations             (Saad Alg. 9.5)
// The triangular sweeps keep the natural row order of the reference's sweeps
// (same operations per row as the CPU code), made parallel by level scheduling:
// the rows of one level are independent and a grid barrier separates levels
// (SellDev::lev; 209 forward levels for the 2M-cell tet cavity).  GMRES
// orthogonalises by classical Gram-Schmidt applied twice (two grid reductions
// per step instead of j + 2 for modified Gram-Schmidt), with exact
// deterministic multi-value grid sums (exact_sum.cuh).
#include "krylov_dev.cuh"

namespace sysu {
namespace {

constexpr int GM_THREADS = 256;
constexpr int GM_WARPS = GM_THREADS / 32;
constexpr int GM_MAXD = GMRES_MAX_RESTART + 2;  // values of one multi-value reduction

struct Pre {
    SellView A;        // the matrix (FP64 values)
    const double *ilu; // ILU(0) factors in A's layout
    const double *dinv;
    int kind;
    double omega;
    const int *fptr, *frows, *bptr, *brows;
    const int4 *finfo, *binfo;
    int nf, nb;
};

// warp-level partial sums of the running reduction, per value and warp
__shared__ long long g_md[GM_MAXD * GM_WARPS * 4];
__shared__ double g_mout[GM_MAXD];

// Exact sums over all rows of nd per-row quantities: f(k, i) for k < nd.
// Every thread gets the totals in g_mout[0..nd).  Threads own rows
// i = gtid, gtid + T, ... (the same rows in every phase of these kernels).
template <class F>
__device__ bool grid_dots(int nd, F f, int n, long long *gpart, int &parity, GridBarrier *gb, int *err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int T = gridDim.x * blockDim.x;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int k = 0; k < nd; ++k) {
        double acc = 0.0;
        for (int i = gtid; i < n; i += T) acc += f(k, i);
        int E, nf;
        I128 S;
        xs_warp(acc, E, S, nf);
        if (lane == 0) {
            long long *q = g_md + (k * GM_WARPS + warp) * 4;
            q[0] = E;
            q[1] = (long long)S.lo;
            q[2] = S.hi;
            q[3] = nf;
        }
    }
    __syncthreads();
    long long *buf = gpart + (size_t)parity * GM_MAXD * gridDim.x * 4;
    parity ^= 1;
    if (warp == 0) {
        for (int k = 0; k < nd; ++k) {
            int e = 0, fl = 0;
            I128 s{0ull, 0ll};
            if (lane < GM_WARPS) {
                const long long *q = g_md + (k * GM_WARPS + lane) * 4;
                e = (int)q[0];
                s.lo = (unsigned long long)q[1];
                s.hi = q[2];
                fl = (int)q[3];
            }
            int E, nf;
            I128 S;
            xs_combine(e, s, fl, 0, E, S, nf);
            if (lane == 0) {
                long long *o = buf + ((size_t)k * gridDim.x + blockIdx.x) * 4;
                o[0] = E;
                o[1] = (long long)S.lo;
                o[2] = S.hi;
                o[3] = nf;
            }
        }
    }
    if (!grid_sync(gb, err)) return false;
    if (warp == 0) {
        for (int k = 0; k < nd; ++k) {
            const long long *pk = buf + (size_t)k * gridDim.x * 4;
            int em = 0;
            for (int b = lane; b < (int)gridDim.x; b += 32) {
                long long lo = __ldcg(pk + b * 4 + 1), hi = __ldcg(pk + b * 4 + 2);
                if (lo != 0 || hi != 0) em = max(em, (int)__ldcg(pk + b * 4));
            }
            int E = __reduce_max_sync(FULL_MASK, em);
            I128 t{0ull, 0ll};
            int fl = 0;
            for (int b = lane; b < (int)gridDim.x; b += 32) {
                I128 sb{(unsigned long long)__ldcg(pk + b * 4 + 1), __ldcg(pk + b * 4 + 2)};
                fl |= (int)__ldcg(pk + b * 4 + 3);
                if (sb.lo != 0 || sb.hi != 0) t = xs_add(t, xs_sar(sb, E - (int)__ldcg(pk + b * 4) + XS_G));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t = xs_add(t, xs_shfl_xor(t, o));
            int nfl = __reduce_or_sync(FULL_MASK, fl);
            double v = xs_to_double(E, t, nfl, XS_G);
            if (lane == 0) g_mout[k] = v;
        }
    }
    __syncthreads();
    return true;
}

// One SELL row: y = sum_k a_k x[col_k] over the row's stored entries.
__device__ __forceinline__ double sell_row(const SellView &A, const double *__restrict__ val, int i,
                                           const double *x) {
    int s = i >> 5;
    int e = __ldg(A.sl_ptr + s) + (i & 31);
    int w = __ldg(A.sl_w + s);
    double acc = 0.0;
    for (int k = 0; k < w; ++k, e += 32) acc = fma(val[e], x[A.col[e]], acc);
    return acc;
}

// Row updates of the triangular sweeps.  (i, e, w) = row, SELL position of its
// entry 0, slice width (one 16-byte load from the level schedule).  Rows of up
// to 8 stored entries load all their columns and values first and then gather
// y, so a row costs two dependent load rounds; the arithmetic and its order are
// those of the plain loop.
#define SWEEP_ROW(COND, COEF, ARR)                                                              \
    if (w <= 8) {                                                                              \
        int jj[8];                                                                             \
        double aa[8];                                                                          \
        _Pragma("unroll") for (int k = 1; k < 8; ++k) if (k < w) {                            \
            jj[k] = P.A.col[e + 32 * k];                                                       \
            aa[k] = ARR[e + 32 * k];                                                           \
        }                                                                                      \
        _Pragma("unroll") for (int k = 1; k < 8; ++k) if (k < w) {                            \
            int j = jj[k];                                                                     \
            if (COND) acc -= COEF aa[k] * y[j];                                                \
        }                                                                                      \
    } else {                                                                                   \
        for (int k = 1; k < w; ++k) {                                                          \
            int j = P.A.col[e + 32 * k];                                                       \
            if (COND) acc -= COEF ARR[e + 32 * k] * y[j];                                     \
        }                                                                                      \
    }

// Forward sweep of SSOR for one row: y_i = (f c_i - w sum_{j<i} a_ij y_j) / a_ii.
__device__ __forceinline__ void ssor_fwd_row(const Pre &P, int i, int e, int w, double f, const double *c,
                                             double *y) {
    double d = P.A.val[e];
    double acc = f * c[i];
    SWEEP_ROW(j < i, P.omega *, P.A.val)
    y[i] = acc / d;
}

// Backward sweep: y_i = (a_ii y_i - w sum_{j>i} a_ij y_j) / a_ii.
__device__ __forceinline__ void ssor_bwd_row(const Pre &P, int i, int e, int w, double *y) {
    double d = P.A.val[e];
    double acc = d * y[i];
    SWEEP_ROW(j > i, P.omega *, P.A.val)
    y[i] = acc / d;
}

// ILU(0) apply rows: forward L y = c (unit diagonal), backward U y = y.
__device__ __forceinline__ void ilu_fwd_row(const Pre &P, int i, int e, int w, const double *c, double *y) {
    double acc = c[i];
    SWEEP_ROW(j < i, , P.ilu)
    y[i] = acc;
}

__device__ __forceinline__ void ilu_bwd_row(const Pre &P, int i, int e, int w, double *y) {
    double acc = y[i];
    SWEEP_ROW(j > i, , P.ilu)
    y[i] = acc / P.ilu[e];
}
#undef SWEEP_ROW

// ILU(0) factorisation of row i (IKJ): its lower entries in ascending column
// order, each eliminating with the already factorised row j.  Entries k >= 1
// whose column is the row itself are SELL padding (value 0) and never match.
// Rows up to 16 entries; *bad set on a zero pivot or a longer row.
__device__ void ilu_factor_row(const Pre &P, double *ilu, int i, int *bad) {
    constexpr int MAXR = 16;
    int s = i >> 5;
    int e = __ldg(P.A.sl_ptr + s) + (i & 31);
    int w = __ldg(P.A.sl_w + s);
    if (w > MAXR) {
        atomicExch(bad, 1);
        return;
    }
    int cols[MAXR];
    double v[MAXR];
    for (int k = 0; k < w; ++k) {
        cols[k] = P.A.col[e + 32 * k];
        v[k] = P.A.val[e + 32 * k];
    }
    int last = -1;
    for (;;) {
        // next lower column in ascending order
        int kj = -1, j = i;
        for (int k = 1; k < w; ++k)
            if (cols[k] < i && cols[k] > last && cols[k] < j) { j = cols[k]; kj = k; }
        if (kj < 0) break;
        last = j;
        int sj = j >> 5;
        int ej = __ldg(P.A.sl_ptr + sj) + (j & 31);
        int wj = __ldg(P.A.sl_w + sj);
        double lij = v[kj] / ilu[ej];
        v[kj] = lij;
        for (int kk = 1; kk < wj; ++kk) {
            int m = P.A.col[ej + 32 * kk];
            if (m <= j) continue;  // row j's upper part only
            double u = ilu[ej + 32 * kk];
            if (m == i) {
                v[0] -= lij * u;
            } else {
                for (int k = 1; k < w; ++k)
                    if (cols[k] == m) v[k] -= lij * u;
            }
        }
    }
    if (v[0] == 0.0) atomicExch(bad, 1);
    for (int k = 0; k < w; ++k) ilu[e + 32 * k] = v[k];
}

// y = M^-1 c by all threads of the grid.  Jacobi and none are row-local (rows
// i = gtid, gtid + T, ..., the rows each thread owns everywhere in these
// kernels).  SSOR and ILU move data between rows: they start with a grid
// barrier (c was written by the rows' owners) and end with one.
__device__ bool precond_dev(const Pre &P, int n, const double *c, double *y, GridBarrier *gb, int *err) {
    const int T = gridDim.x * blockDim.x;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    if (P.kind == PK_NONE) {
        for (int i = gtid; i < n; i += T) y[i] = c[i];
        return true;
    }
    if (P.kind == PK_JACOBI) {
        for (int i = gtid; i < n; i += T) y[i] = P.dinv[i] * c[i];
        return true;
    }
    if (!grid_sync(gb, err)) return false;
    if (P.kind == PK_SSOR) {
        const double f = P.omega * (2.0 - P.omega);
        for (int l = 0; l < P.nf; ++l) {
            for (int r = P.fptr[l] + gtid; r < P.fptr[l + 1]; r += T) {
                int4 q = P.finfo[r];
                ssor_fwd_row(P, q.x, q.y, q.z, f, c, y);
            }
            if (!grid_sync(gb, err)) return false;
        }
        for (int l = 0; l < P.nb; ++l) {
            for (int r = P.bptr[l] + gtid; r < P.bptr[l + 1]; r += T) {
                int4 q = P.binfo[r];
                ssor_bwd_row(P, q.x, q.y, q.z, y);
            }
            if (!grid_sync(gb, err)) return false;
        }
        return true;
    }
    // ILU(0)
    for (int l = 0; l < P.nf; ++l) {
        for (int r = P.fptr[l] + gtid; r < P.fptr[l + 1]; r += T) {
            int4 q = P.finfo[r];
            ilu_fwd_row(P, q.x, q.y, q.z, c, y);
        }
        if (!grid_sync(gb, err)) return false;
    }
    for (int l = 0; l < P.nb; ++l) {
        for (int r = P.bptr[l] + gtid; r < P.bptr[l + 1]; r += T) {
            int4 q = P.binfo[r];
            ilu_bwd_row(P, q.x, q.y, q.z, y);
        }
        if (!grid_sync(gb, err)) return false;
    }
    return true;
}

// Factorise ILU(0) (level by level) when the preconditioner is ILU.
__device__ bool precond_setup(const Pre &P, double *ilu, GridBarrier *gb, int *err, int *bad) {
    if (P.kind != PK_ILU0) return true;
    const int T = gridDim.x * blockDim.x;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int l = 0; l < P.nf; ++l) {
        for (int r = P.fptr[l] + gtid; r < P.fptr[l + 1]; r += T) ilu_factor_row(P, ilu, P.frows[r], bad);
        if (!grid_sync(gb, err)) return false;
    }
    return true;
}

struct GmArgs {
    Pre P;
    double *ilu;
    const double *b;
    double *x;
    double *V, *Z, *w;
    long long *gpart;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit, m;
    double eps;
};

__global__ void __launch_bounds__(GM_THREADS) k_gmres(GmArgs a) {
    const int n = a.P.A.n;
    const int T = gridDim.x * blockDim.x;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    int *err = &a.info->err;
    int parity = 0;
    const int m = a.m;
    __shared__ double H[(GMRES_MAX_RESTART + 1) * GMRES_MAX_RESTART];
    __shared__ double cs[GMRES_MAX_RESTART], sn[GMRES_MAX_RESTART], g[GMRES_MAX_RESTART + 1],
        yv[GMRES_MAX_RESTART];
    int status = DEV_OK;
    if (!precond_setup(a.P, a.ilu, a.gb, err, &a.info->status[1])) return;
    const SellView &A = a.P.A;
    // ||b||
    if (!grid_dots(1, [&](int, int i) { return a.b[i] * a.b[i]; }, n, a.gpart, parity, a.gb, err)) return;
    double bnorm = sqrt(g_mout[0]);
    if (bnorm == 0.0) bnorm = 1.0;
    int it = 0;
    double res = 0.0;
    for (;;) {
        // v0 = b - A x, beta = ||v0||
        for (int i = gtid; i < n; i += T) a.V[i] = a.b[i] - sell_row(A, A.val, i, a.x);
        if (!grid_dots(1, [&](int, int i) { return a.V[i] * a.V[i]; }, n, a.gpart, parity, a.gb, err)) return;
        double beta = sqrt(g_mout[0]);
        res = beta / bnorm;
        if (res < a.eps || it >= a.maxit || beta == 0.0) break;
        if (!isfinite(res)) { status = DEV_NONFINITE; break; }
        for (int i = gtid; i < n; i += T) a.V[i] /= beta;
        if (threadIdx.x == 0) {
            for (int k = 0; k <= m; ++k) g[k] = 0.0;
            g[0] = beta;
        }
        int j = 0;
        for (; j < m && it < a.maxit; ++j) {
            ++it;
            const double *vj = a.V + (size_t)j * n;
            double *zj = a.Z + (size_t)j * n;
            if (!precond_dev(a.P, n, vj, zj, a.gb, err)) return;
            if (!grid_sync(a.gb, err)) return;  // z_j complete before the product
            for (int i = gtid; i < n; i += T) a.w[i] = sell_row(A, A.val, i, zj);
            // classical Gram-Schmidt, pass 1: h_k = w . v_k, w -= sum h_k v_k
            if (!grid_dots(j + 1, [&](int k, int i) { return a.w[i] * a.V[(size_t)k * n + i]; }, n, a.gpart,
                           parity, a.gb, err))
                return;
            if (threadIdx.x == 0)
                for (int k = 0; k <= j; ++k) H[k * m + j] = g_mout[k];
            for (int i = gtid; i < n; i += T) {
                double wi = a.w[i];
                for (int k = 0; k <= j; ++k) wi -= g_mout[k] * a.V[(size_t)k * n + i];
                a.w[i] = wi;
            }
            __syncthreads();  // g_mout is rewritten by the next reduction
            // pass 2 (re-orthogonalisation) and ||w||^2 in the same reduction
            if (!grid_dots(j + 2,
                           [&](int k, int i) {
                               double wi = a.w[i];
                               return k <= j ? wi * a.V[(size_t)k * n + i] : wi * wi;
                           },
                           n, a.gpart, parity, a.gb, err))
                return;
            // ||w - sum h2_k v_k||^2 = ||w||^2 - sum h2_k^2 (v_k orthonormal)
            double hn2 = g_mout[j + 1];
            for (int k = 0; k <= j; ++k) hn2 -= g_mout[k] * g_mout[k];
            double hn = sqrt(fmax(hn2, 0.0));
            double *vn = a.V + (size_t)(j + 1) * n;
            for (int i = gtid; i < n; i += T) {
                double wi = a.w[i];
                for (int k = 0; k <= j; ++k) wi -= g_mout[k] * a.V[(size_t)k * n + i];
                vn[i] = hn != 0.0 ? wi / hn : 0.0;
            }
            if (threadIdx.x == 0) {
                for (int k = 0; k <= j; ++k) H[k * m + j] += g_mout[k];
                H[(j + 1) * m + j] = hn;
                for (int k = 0; k < j; ++k) {
                    double a0 = H[k * m + j], c2 = H[(k + 1) * m + j];
                    H[k * m + j] = cs[k] * a0 + sn[k] * c2;
                    H[(k + 1) * m + j] = -sn[k] * a0 + cs[k] * c2;
                }
                double a0 = H[j * m + j], c2 = H[(j + 1) * m + j];
                double den = sqrt(a0 * a0 + c2 * c2);
                cs[j] = den != 0.0 ? a0 / den : 1.0;
                sn[j] = den != 0.0 ? c2 / den : 0.0;
                H[j * m + j] = den;
                H[(j + 1) * m + j] = 0.0;
                g[j + 1] = -sn[j] * g[j];
                g[j] = cs[j] * g[j];
                g_bc[0] = fabs(g[j + 1]) / bnorm;
                g_bc[1] = hn == 0.0 ? 1.0 : 0.0;
            }
            __syncthreads();
            res = g_bc[0];
            bool brk = g_bc[1] != 0.0;
            __syncthreads();
            if (res < a.eps || brk) {
                ++j;
                break;
            }
        }
        // y = H^-1 g (back substitution), x += sum y_k z_k
        if (threadIdx.x == 0) {
            for (int k = j - 1; k >= 0; --k) {
                double sacc = g[k];
                for (int l = k + 1; l < j; ++l) sacc -= H[k * m + l] * yv[l];
                yv[k] = sacc / H[k * m + k];
            }
        }
        __syncthreads();
        for (int i = gtid; i < n; i += T) {
            double xi = a.x[i];
            for (int k = 0; k < j; ++k) xi += yv[k] * a.Z[(size_t)k * n + i];
            a.x[i] = xi;
        }
        if (!grid_sync(a.gb, err)) return;  // x complete before the residual of the next cycle
        if (res < a.eps || it >= a.maxit) {
            // the oracle checks the true residual before it stops
            for (int i = gtid; i < n; i += T) a.w[i] = a.b[i] - sell_row(A, A.val, i, a.x);
            if (!grid_dots(1, [&](int, int i) { return a.w[i] * a.w[i]; }, n, a.gpart, parity, a.gb, err)) return;
            res = sqrt(g_mout[0]) / bnorm;
            if (res < a.eps || it >= a.maxit) break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.info->status[1]) status = DEV_BREAKDOWN;  // ILU zero pivot
        if (status == DEV_OK && !(res < a.eps)) status = isfinite(res) ? DEV_MAXITER : DEV_NONFINITE;
        a.info->status[0] = status;
        a.info->iters[0] = it;
        a.info->res[0] = res;
    }
}

struct PcgArgs {
    Pre P;
    double *ilu;
    const double *b;
    double *x, *r, *z, *p, *q;
    long long *gpart;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit;
    double eps;
};

__global__ void __launch_bounds__(GM_THREADS) k_pcg(PcgArgs a) {
    const int n = a.P.A.n;
    const int T = gridDim.x * blockDim.x;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    int *err = &a.info->err;
    int parity = 0;
    if (!precond_setup(a.P, a.ilu, a.gb, err, &a.info->status[1])) return;
    const SellView &A = a.P.A;
    for (int i = gtid; i < n; i += T) a.r[i] = a.b[i] - sell_row(A, A.val, i, a.x);
    if (!grid_dots(2, [&](int k, int i) { return k == 0 ? a.b[i] * a.b[i] : a.r[i] * a.r[i]; }, n, a.gpart,
                   parity, a.gb, err))
        return;
    double bb = g_mout[0] == 0.0 ? 1.0 : g_mout[0];
    double rr = g_mout[1];
    const double thr = a.eps * a.eps * bb;
    double rho_prev = 1.0;
    int it = 0, status = DEV_OK;
    for (;;) {
        if (rr < thr || it >= a.maxit) break;
        if (!isfinite(rr)) { status = DEV_NONFINITE; break; }
        ++it;
        if (!precond_dev(a.P, n, a.r, a.z, a.gb, err)) return;
        if (!grid_dots(1, [&](int, int i) { return a.r[i] * a.z[i]; }, n, a.gpart, parity, a.gb, err)) return;
        double rho = g_mout[0];
        double beta = it == 1 ? 0.0 : rho / rho_prev;
        for (int i = gtid; i < n; i += T) a.p[i] = it == 1 ? a.z[i] : fma(beta, a.p[i], a.z[i]);
        if (!grid_sync(a.gb, err)) return;
        for (int i = gtid; i < n; i += T) a.q[i] = sell_row(A, A.val, i, a.p);
        if (!grid_dots(1, [&](int, int i) { return a.p[i] * a.q[i]; }, n, a.gpart, parity, a.gb, err)) return;
        double pq = g_mout[0];
        if (pq == 0.0) { status = DEV_BREAKDOWN; break; }
        double alpha = rho / pq;
        for (int i = gtid; i < n; i += T) {
            a.x[i] = fma(alpha, a.p[i], a.x[i]);
            a.r[i] = fma(-alpha, a.q[i], a.r[i]);
        }
        if (!grid_dots(1, [&](int, int i) { return a.r[i] * a.r[i]; }, n, a.gpart, parity, a.gb, err)) return;
        rr = g_mout[0];
        rho_prev = rho;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.info->status[1]) status = DEV_BREAKDOWN;
        if (status == DEV_OK && !(rr < thr)) status = isfinite(rr) ? DEV_MAXITER : DEV_NONFINITE;
        a.info->status[0] = status;
        a.info->iters[0] = it;
        a.info->res[0] = sqrt(rr) / sqrt(bb);
    }
}

struct PcArgs {
    Pre P;
    double *ilu;
    const double *c;
    double *y;
    GridBarrier *gb;
    SolveInfo *info;
};

__global__ void __launch_bounds__(GM_THREADS) k_precond_once(PcArgs a) {
    int *err = &a.info->err;
    if (!precond_setup(a.P, a.ilu, a.gb, err, &a.info->status[1])) return;
    precond_dev(a.P, a.P.A.n, a.c, a.y, a.gb, err);
}

__global__ void k_dinv_omega(SellView A, double omega, double *dinv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    dinv[i] = omega / A.val[A.sl_ptr[i >> 5] + (i & 31)];
}

template <class K>
int gm_blocks(K kernel, int n) {
    int per_sm = 0;
    SYSU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, GM_THREADS, 0));
    if (per_sm < 1) throw CaseError{"persistent Krylov kernel cannot be resident"};
    int want = (n + GM_THREADS - 1) / GM_THREADS;
    return std::max(1, std::min(want, per_sm * num_sms()));
}

Pre make_pre(const SellDev &A, const double *val, int precond, double omega, KrylovWork &w, cudaStream_t st) {
    if (precond < PK_NONE || precond > PK_ILU0) throw CaseError{"unknown preconditioner"};
    Pre P{};
    P.A = view(A, val);
    P.kind = precond;
    P.omega = omega;
    P.fptr = A.lev.fptr.get();
    P.frows = A.lev.frows.get();
    P.bptr = A.lev.bptr.get();
    P.brows = A.lev.brows.get();
    P.finfo = A.lev.finfo.get();
    P.binfo = A.lev.binfo.get();
    P.nf = A.lev.nf;
    P.nb = A.lev.nb;
    if (precond == PK_JACOBI) {
        { k_dinv_omega<<<(A.n + KB - 1) / KB, KB, 0, st>>>(P.A, omega, w.dinv.get()); ++::sysu::g_launches; }
        P.dinv = w.dinv.get();
    }
    if (precond == PK_ILU0) {
        if (w.ilu.size() < (size_t)A.nnz) w.ilu.alloc(A.nnz);
        P.ilu = w.ilu.get();
    }
    return P;
}

void ensure_general(KrylovWork &w, int n, int m, int blocks, cudaStream_t st) {
    w.ensure(n, 1, std::max(blocks, w.max_blocks), st);
    size_t need_v = (size_t)(m + 1) * n, need_z = (size_t)m * n;
    if (w.gV.size() < need_v) w.gV.alloc(need_v);
    if (w.gZ.size() < need_z) w.gZ.alloc(need_z);
    if (w.gW.size() < (size_t)n) w.gW.alloc(n);
    size_t need_p = (size_t)2 * GM_MAXD * blocks * 4;
    if (w.gpart.size() < need_p) w.gpart.alloc(need_p);
}

}  // namespace

void gmres_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
                 const KrylovOpts &o, int precond, int restart, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    if (restart < 1 || restart > GMRES_MAX_RESTART) throw CaseError{"GMRES restart length must be 1..30"};
    static int maxb = 0;
    if (!maxb) maxb = gm_blocks(k_gmres, 1 << 30);
    int G = std::max(1, std::min((n + GM_THREADS - 1) / GM_THREADS, maxb));
    ensure_general(w, n, restart, G, st);
    if (x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    GmArgs a{};
    a.P = make_pre(A, val, precond, o.omega, w, st);
    a.ilu = w.ilu.get();
    a.b = b;
    a.x = x;
    a.V = w.gV.get();
    a.Z = w.gZ.get();
    a.w = w.gW.get();
    a.gpart = w.gpart.get();
    a.gb = w.barrier.get();
    a.info = info;
    a.maxit = o.maxit;
    a.m = restart;
    a.eps = o.eps;
    void *args[] = {&a};
    SYSU_CUDA(cudaMemsetAsync(w.barrier.get(), 0, sizeof(GridBarrier), st));  // grid_sync starts from 0
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_gmres, dim3(G), dim3(GM_THREADS), args, 0, st)); ++::sysu::g_launches; }
}

void pcg_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero, const KrylovOpts &o,
               int precond, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = gm_blocks(k_pcg, 1 << 30);
    int G = std::max(1, std::min((n + GM_THREADS - 1) / GM_THREADS, maxb));
    ensure_general(w, n, 1, G, st);
    if (x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    PcgArgs a{};
    a.P = make_pre(A, val, precond, o.omega, w, st);
    a.ilu = w.ilu.get();
    a.b = b;
    a.x = x;
    a.r = w.r.get();
    a.z = w.s.get();
    a.p = w.p.get();
    a.q = w.v.get();
    a.gpart = w.gpart.get();
    a.gb = w.barrier.get();
    a.info = info;
    a.maxit = o.maxit;
    a.eps = o.eps;
    void *args[] = {&a};
    SYSU_CUDA(cudaMemsetAsync(w.barrier.get(), 0, sizeof(GridBarrier), st));  // grid_sync starts from 0
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_pcg, dim3(G), dim3(GM_THREADS), args, 0, st)); ++::sysu::g_launches; }
}

void precond_solve(const SellDev &A, const double *val, int precond, double omega, const double *c, double *y,
                   KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = gm_blocks(k_precond_once, 1 << 30);
    int G = std::max(1, std::min((n + GM_THREADS - 1) / GM_THREADS, maxb));
    ensure_general(w, n, 1, G, st);
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    PcArgs a{};
    a.P = make_pre(A, val, precond, omega, w, st);
    a.ilu = w.ilu.get();
    a.c = c;
    a.y = y;
    a.gb = w.barrier.get();
    a.info = info;
    void *args[] = {&a};
    SYSU_CUDA(cudaMemsetAsync(w.barrier.get(), 0, sizeof(GridBarrier), st));  // grid_sync starts from 0
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_precond_once, dim3(G), dim3(GM_THREADS), args, 0, st)); ++::sysu::g_launches; }
}

}  // namespace sysu
