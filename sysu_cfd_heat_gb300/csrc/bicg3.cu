// Momentum u, v, w by one BiCGSTAB + Jacobi sequence with FP32 recurrences and
// FP64 residual replacement (the FP64 form is k_bicgstab<3, false>, which
// replaces BiCGSTABIter as called from navier_velocity.cpp:26 for each
// component).
//
// The three systems share the momentum matrix.  Their vectors are interleaved
// per row as float4 (u, v, w, spare), so one matrix read and one 16-byte gather
// per entry serve all three products, and the vector passes are unit-stride
// 16-byte loads.  The spare lane of the shadow residual holds the row's FP32
// Jacobi weight, which the x update reads with it.
//
// Per component c the recurrences run on the preconditioned correction
// equation in units of sig_c (a power of two, sig_c ||r_c|| ~ 1 at the last
// replacement): the matrix is the FP32 column-scaled a_ij d_j, the scalars
// (alpha, omega, rho, beta) are FP64 from FP64 grid sums of per-thread FP32
// partials.  Every iteration adds its correction d (alpha p + omega s) to an
// FP32 accumulator e.  When the FP32 residual has fallen by inner_tol since the
// last replacement (or below the stopping threshold, or at the iteration cap),
// x += e / sig in FP64, the FP64 residual b - A x replaces r and the
// convergence test ||b - A x|| / ||b|| < eps is made on it;
// the recurrences continue (rho is recomputed on the replaced r, which folds a
// change of sig into beta exactly).  A breakdown (rt.v = 0, omega = 0, rho =
// 0) or a small s (the FP64 method's early exit) restarts component c from its
// replaced residual (rt = r, p = r).  Three replacements without a lower FP64
// residual stop the component as stalled, and the FP64 solve finishes it from
// its x.
//
// Each phase is one flat kernel over all rows; the last block to finish a
// phase reduces the partial sums (fixed order: run-to-run deterministic) and
// derives the next scalars into the device state.  CH iterations are the body
// of a CUDA graph WHILE node whose last kernel ends the loop (graph_loop.hpp);
// the FP64 finish of stalled components is an IF node.  The solve never waits
// for the host (device_loop false: the host drives the same body, for
// per-kernel profiling).
#include <cstring>

#include "graph_loop.hpp"
#include "krylov_dev.cuh"

namespace sysu {
namespace {

constexpr int MB = 256;  // threads per block
constexpr int CH = 4;    // iterations per captured graph

struct M3State {
    double bb[3], thr[3], sig[3], sig_next[3], rr64[3], best64[3];
    double rho[3], rho_prev[3], alpha[3], omg[3], beta[3], rref[3];
    int it[3], status[3], done[3], need[3], restart[3], skip[3], early[3], upd[3], stall[3];
    int all_done, any_need, maxit;
    int loops;    // graph loop: bodies run (the loop's bound)
    int stalled;  // a component handed to the FP64 solve
    double d2;
    // arrival count of grid_sums: the phases run one after another on one
    // stream, and the last block resets it before its kernel ends
    unsigned cnt;
};

struct M3Args {
    int n;
    const int *sl_ptr, *sl_w, *col;
    float *sv;          // FP32 column-scaled values a_ij d_j
    const double *val;  // FP64 values (residual replacement)
    float *dinv;        // FP32 Jacobi weights
    double *r0;         // the FP64 residual of x0 (three arrays of n), from k_m3_init
    const double *b[3];
    double *x[3];
    float4 *r, *rtd, *p, *v, *s, *t, *e;
    M3State *st;
    double *part;
};

__device__ __forceinline__ float &comp(float4 &a, int c) { return c == 0 ? a.x : (c == 1 ? a.y : a.z); }
__device__ __forceinline__ float comp(const float4 &a, int c) { return c == 0 ? a.x : (c == 1 ? a.y : a.z); }

// y = A_s x for the three interleaved components of one SELL row; four
// entries' loads are issued before their FMAs
__device__ __forceinline__ float4 row3(const M3Args &a, int i, const float4 *__restrict__ x) {
    const int sl = i >> 5;
    int e = a.sl_ptr[sl] + (i & 31);
    const int w = a.sl_w[sl];
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    int k = 0;
    for (; k + 4 <= w; k += 4, e += 128) {
        const int c0 = __ldg(a.col + e), c1 = __ldg(a.col + e + 32), c2 = __ldg(a.col + e + 64),
                  c3 = __ldg(a.col + e + 96);
        const float v0 = __ldg(a.sv + e), v1 = __ldg(a.sv + e + 32), v2 = __ldg(a.sv + e + 64),
                    v3 = __ldg(a.sv + e + 96);
        const float4 x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
        y0 = fmaf(v0, x0.x, y0); y1 = fmaf(v0, x0.y, y1); y2 = fmaf(v0, x0.z, y2);
        y0 = fmaf(v1, x1.x, y0); y1 = fmaf(v1, x1.y, y1); y2 = fmaf(v1, x1.z, y2);
        y0 = fmaf(v2, x2.x, y0); y1 = fmaf(v2, x2.y, y1); y2 = fmaf(v2, x2.z, y2);
        y0 = fmaf(v3, x3.x, y0); y1 = fmaf(v3, x3.y, y1); y2 = fmaf(v3, x3.z, y2);
    }
    for (; k < w; ++k, e += 32) {
        const float vk = __ldg(a.sv + e);
        const float4 xk = __ldg(x + __ldg(a.col + e));
        y0 = fmaf(vk, xk.x, y0); y1 = fmaf(vk, xk.y, y1); y2 = fmaf(vk, xk.z, y2);
    }
    return make_float4(y0, y1, y2, 0.f);
}

// b_c - A x_c in FP64 for the components with want[c]; four entries' loads
// are issued before their FMAs
__device__ __forceinline__ void resid3(const M3Args &a, int i, const bool (&want)[3], double (&r)[3]) {
    const int sl = i >> 5;
    int e = a.sl_ptr[sl] + (i & 31);
    const int w = a.sl_w[sl];
    double y[3] = {0.0, 0.0, 0.0};
    int k = 0;
    for (; k + 4 <= w; k += 4, e += 128) {
        int j[4];
        double v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            j[q] = __ldg(a.col + e + 32 * q);
            v[q] = __ldg(a.val + e + 32 * q);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (!want[c]) continue;
            const double *xc = a.x[c];
            const double x0 = xc[j[0]], x1 = xc[j[1]], x2 = xc[j[2]], x3 = xc[j[3]];
            y[c] = fma(v[0], x0, y[c]);
            y[c] = fma(v[1], x1, y[c]);
            y[c] = fma(v[2], x2, y[c]);
            y[c] = fma(v[3], x3, y[c]);
        }
    }
    for (; k < w; ++k, e += 32) {
        const int j = __ldg(a.col + e);
        const double vk = __ldg(a.val + e);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (want[c]) y[c] = fma(vk, a.x[c][j], y[c]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] = want[c] ? a.b[c][i] - y[c] : 0.0;
}

// Jacobi weights in FP32, d_i = omega / a_ii (1 without a preconditioner); the
// diagonal is entry 0 of every row
__global__ void __launch_bounds__(MB) k_m3_dinv(M3Args a, float omega, int jacobi) {
    const int i = blockIdx.x * MB + threadIdx.x;
    if (i >= a.n) return;
    a.dinv[i] = jacobi ? omega / (float)a.val[a.sl_ptr[i >> 5] + (i & 31)] : 1.f;
}

// The operator of the FP32 recurrences: sv_e = a_e d_(col e) in FP32 over all
// stored entries (padding entries hold 0)
__global__ void __launch_bounds__(MB) k_m3_scale(M3Args a, long nnz) {
    const long e = (long)blockIdx.x * MB + threadIdx.x;
    if (e < nnz) a.sv[e] = (float)a.val[e] * a.dinv[a.col[e]];
}

// First pass: ||b||^2 and ||b - A x0||^2 per component (the residual kept in r0
// for the set-up replacement), the scale of the FP32 vectors, and the vectors'
// initial contents (rtd = (0, 0, 0, d), p = v = e = 0).
__global__ void __launch_bounds__(MB) k_m3_init(M3Args a, int maxit, double eps, double d2) {
    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const bool all[3] = {true, true, true};
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        double r[3];
        resid3(a, i, all, r);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double bi = a.b[c][i];
            v[c] = fma(bi, bi, v[c]);
            v[3 + c] = fma(r[c], r[c], v[3 + c]);
            a.r0[(size_t)c * a.n + i] = r[c];
        }
        a.rtd[i] = make_float4(0.f, 0.f, 0.f, a.dinv[i]);
        a.p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.e[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (!grid_sums<6>(v, a.part, &a.st->cnt)) return;
    M3State *S = a.st;
    S->maxit = maxit;
    S->d2 = d2;
    int need = 0, all_done = 1;
    for (int c = 0; c < 3; ++c) {
        S->bb[c] = v[c] == 0.0 ? 1.0 : v[c];
        S->thr[c] = eps * eps * S->bb[c];
        S->rr64[c] = S->best64[c] = v[3 + c];
        S->sig_next[c] = pow2_scale(v[3 + c]);
        S->sig[c] = S->sig_next[c];
        S->it[c] = S->upd[c] = S->stall[c] = 0;
        S->skip[c] = S->early[c] = 0;
        S->status[c] = DEV_OK;
        S->rho[c] = S->rho_prev[c] = S->alpha[c] = S->omg[c] = 1.0;
        S->beta[c] = 0.0;
        S->rref[c] = 1.0;
        const double rr = v[3 + c];
        S->done[c] = !isfinite(rr) ? 1 : (rr < S->thr[c] ? 1 : 0);
        if (!isfinite(rr)) S->status[c] = DEV_NONFINITE;
        else if (!S->done[c] && maxit <= 0) { S->done[c] = 1; S->status[c] = DEV_MAXITER; }
        S->need[c] = S->restart[c] = !S->done[c];
        need |= S->need[c];
        all_done &= S->done[c];
    }
    S->any_need = need;
    S->all_done = all_done;
}

// FP64 residual replacement for the components that need it: r_c = sig (b - A x)
// with the scale chosen from the FP32 residual that triggered it; rt_c = r_c
// when the component restarts.  first: the set-up pass (the residual of x0 from
// r0, no stall bookkeeping).
__global__ void __launch_bounds__(MB) k_m3_replace(M3Args a, int first) {
    const M3State *S = a.st;
    if (S->all_done || !S->any_need) return;
    bool want[3], rs[3];
    double sg[3];
    bool any_rs = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        want[c] = S->need[c] && !S->done[c];
        rs[c] = want[c] && S->restart[c];
        any_rs |= rs[c];
        sg[c] = S->sig_next[c];
    }
    // the norms come from the scaled FP32 residual (sig r ~ 1: no under- or
    // overflow), summed like the recurrences' dot products; an FP64 square per row
    // and an FP64 shuffle tree would cost a fifth of this FP64-bound pass
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        double r64[3];
        if (first) {
#pragma unroll
            for (int c = 0; c < 3; ++c) r64[c] = want[c] ? a.r0[(size_t)c * a.n + i] : 0.0;
        } else {
            resid3(a, i, want, r64);
        }
        float4 r = a.r[i];
        float4 rt = a.rtd[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (!want[c]) continue;
            const float rn = (float)(sg[c] * r64[c]);
            comp(r, c) = rn;
            if (rs[c]) comp(rt, c) = rn;
            f[c] = fmaf(rn, rn, f[c]);
            f[3 + c] = fmaf(comp(rt, c), rn, f[3 + c]);
        }
        a.r[i] = r;
        if (any_rs) a.rtd[i] = rt;
    }
    double v[6];
    if (!grid_sums_f<6>(f, v, a.part, &a.st->cnt)) return;
    M3State *W = a.st;
    int all_done = 1;
    for (int c = 0; c < 3; ++c) {
        if (want[c]) {
            const double rr = v[c] / (sg[c] * sg[c]);  // ||b - A x||^2
            if (!first) W->upd[c] += 1;
            W->rr64[c] = rr;
            W->sig[c] = W->sig_next[c];
            W->rref[c] = v[c];
            if (rs[c]) {
                W->rho[c] = v[c];
            } else {
                // the recurrences go on with the replaced residual: rho on it; the
                // previous rho is in the old scale, which makes beta carry the
                // change of scale onto the old p - omega v
                W->rho[c] = v[3 + c];
                W->beta[c] = W->omg[c] != 0.0 ? (W->rho[c] / W->rho_prev[c]) * (W->alpha[c] / W->omg[c]) : 0.0;
            }
            if (!first) {
                if (rr < W->best64[c]) {
                    W->best64[c] = rr;
                    W->stall[c] = 0;
                } else {
                    W->stall[c] += 1;
                }
            }
            if (!isfinite(rr)) { W->done[c] = 1; W->status[c] = DEV_NONFINITE; }
            else if (rr < W->thr[c]) W->done[c] = 1;
            else if (W->stall[c] >= 3) { W->done[c] = 1; W->status[c] = DEV_STALLED; }  // FP64 takes over
            else if (W->it[c] >= W->maxit) { W->done[c] = 1; W->status[c] = DEV_MAXITER; }
            W->need[c] = 0;
            W->skip[c] = 0;
        }
        all_done &= W->done[c];
    }
    W->any_need = 0;
    W->all_done = all_done;
}

// p = r (restart) or r + beta (p - omega v)
__global__ void __launch_bounds__(MB) k_m3_dir(M3Args a) {
    const M3State *S = a.st;
    if (S->all_done) return;
    int md[3];
    float bt[3], om[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        md[c] = S->done[c] ? 0 : (S->restart[c] ? 1 : 2);
        bt[c] = (float)S->beta[c];
        om[c] = (float)S->omg[c];
    }
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        const float4 r = a.r[i], v = a.v[i];
        float4 p = a.p[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (md[c] == 1) comp(p, c) = comp(r, c);
            else if (md[c] == 2) comp(p, c) = fmaf(bt[c], fmaf(-om[c], comp(v, c), comp(p, c)), comp(r, c));
        }
        a.p[i] = p;
    }
}

// v = A_s p ; rt.v -> alpha = rho / rt.v
__global__ void __launch_bounds__(MB, 8) k_m3_av(M3Args a) {
    if (a.st->all_done) return;
    float f[3] = {0.f, 0.f, 0.f};
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        const float4 y = row3(a, i, a.p);
        a.v[i] = y;
        const float4 rt = a.rtd[i];
        f[0] = fmaf(rt.x, y.x, f[0]);
        f[1] = fmaf(rt.y, y.y, f[1]);
        f[2] = fmaf(rt.z, y.z, f[2]);
    }
    double v[3];
    if (!grid_sums_f<3>(f, v, a.part, &a.st->cnt)) return;
    M3State *S = a.st;
    for (int c = 0; c < 3; ++c) {
        if (S->done[c]) continue;
        if (v[c] == 0.0 || !isfinite(v[c])) {  // breakdown: replace and restart
            S->skip[c] = 1;
            S->need[c] = 1;
            S->restart[c] = 1;
            S->sig_next[c] = S->sig[c];
            S->any_need = 1;
        } else {
            S->alpha[c] = S->rho[c] / v[c];
        }
    }
}

// s = r - alpha v ; s.s -> early (s small enough for a replacement)
__global__ void __launch_bounds__(MB) k_m3_s(M3Args a) {
    const M3State *S = a.st;
    if (S->all_done) return;
    float al[3];
    bool on[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        on[c] = !S->done[c] && !S->skip[c];
        al[c] = (float)S->alpha[c];
    }
    // s of a component that is done or broke down is never read: every lane is
    // written, only the running ones are summed
    float f[3] = {0.f, 0.f, 0.f};
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        const float4 r = a.r[i], v = a.v[i];
        float4 s;
        s.w = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float si = fmaf(-al[c], comp(v, c), comp(r, c));
            comp(s, c) = si;
            if (on[c]) f[c] = fmaf(si, si, f[c]);
        }
        a.s[i] = s;
    }
    double v[3];
    if (!grid_sums_f<3>(f, v, a.part, &a.st->cnt)) return;
    M3State *W = a.st;
    for (int c = 0; c < 3; ++c) {
        if (!on[c]) continue;
        const double sc2 = W->sig[c] * W->sig[c];
        W->early[c] = v[c] <= W->d2 * W->rref[c] || v[c] < W->thr[c] * sc2;
        if (W->early[c]) W->sig_next[c] = pow2_scale(v[c] / sc2);
    }
}

// t = A_s s ; t.s, t.t -> omega
__global__ void __launch_bounds__(MB, 6) k_m3_at(M3Args a) {
    if (a.st->all_done) return;
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        const float4 y = row3(a, i, a.s);
        a.t[i] = y;
        const float4 s = a.s[i];
        f[0] = fmaf(y.x, s.x, f[0]);
        f[1] = fmaf(y.y, s.y, f[1]);
        f[2] = fmaf(y.z, s.z, f[2]);
        f[3] = fmaf(y.x, y.x, f[3]);
        f[4] = fmaf(y.y, y.y, f[4]);
        f[5] = fmaf(y.z, y.z, f[5]);
    }
    double v[6];
    if (!grid_sums_f<6>(f, v, a.part, &a.st->cnt)) return;
    M3State *S = a.st;
    for (int c = 0; c < 3; ++c)
        if (!S->done[c] && !S->skip[c] && !S->early[c]) S->omg[c] = v[3 + c] != 0.0 ? v[c] / v[3 + c] : 0.0;
}

// e += d (alpha p + omega s) ; r = s - omega t ; r.r, rt.r -> rho, beta, and
// whether a replacement follows
__global__ void __launch_bounds__(MB, 6) k_m3_upd(M3Args a) {
    const M3State *S = a.st;
    if (S->all_done) return;
    bool on[3], ea[3];
    float al[3], om[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        on[c] = !S->done[c] && !S->skip[c];
        ea[c] = S->early[c] != 0;
        al[c] = (float)S->alpha[c];
        om[c] = ea[c] ? 0.f : (float)S->omg[c];
    }
    // r of a component that is done is never read again, and one that exits
    // early or broke down gets its r from the replacement that follows: every
    // lane is written, only the running ones update e and are summed
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        const float4 p = a.p[i], s = a.s[i], t = a.t[i], rtd = a.rtd[i];
        float4 e = a.e[i];
        float4 r;
        r.w = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float ri = fmaf(-om[c], comp(t, c), comp(s, c));
            comp(r, c) = ri;
            if (!on[c]) continue;
            comp(e, c) = fmaf(rtd.w, fmaf(al[c], comp(p, c), om[c] * comp(s, c)), comp(e, c));
            if (ea[c]) continue;
            f[c] = fmaf(ri, ri, f[c]);
            f[3 + c] = fmaf(comp(rtd, c), ri, f[3 + c]);
        }
        a.e[i] = e;
        a.r[i] = r;
    }
    double v[6];
    if (!grid_sums_f<6>(f, v, a.part, &a.st->cnt)) return;
    M3State *W = a.st;
    int need = W->any_need;
    for (int c = 0; c < 3; ++c) {
        if (!on[c]) continue;
        W->it[c] += 1;
        if (ea[c]) {
            W->need[c] = 1;
            W->restart[c] = 1;
            W->early[c] = 0;
        } else {
            const double rr = v[c], sc2 = W->sig[c] * W->sig[c];
            W->rho_prev[c] = W->rho[c];
            W->rho[c] = v[3 + c];
            W->restart[c] = 0;
            const bool brk = W->omg[c] == 0.0 || W->rho[c] == 0.0 || W->rho_prev[c] == 0.0 || !isfinite(rr);
            W->beta[c] = brk ? 0.0 : (W->rho[c] / W->rho_prev[c]) * (W->alpha[c] / W->omg[c]);
            if (brk) {
                W->need[c] = 1;
                W->restart[c] = 1;
            } else if (rr <= W->d2 * W->rref[c] || rr < W->thr[c] * sc2 || W->it[c] >= W->maxit) {
                W->need[c] = 1;
            }
            if (W->need[c]) W->sig_next[c] = isfinite(rr) && rr > 0.0 ? pow2_scale(rr / sc2) : W->sig[c];
        }
        need |= W->need[c];
    }
    // a replacement costs about as much for one component as for three (the
    // matrix pass is shared): a running component whose FP32 residual has fallen
    // by sqrt(inner_tol) since its last replacement is replaced along with the due
    // ones, which saves the pass it would take an iteration or two later
    if (need)
        for (int c = 0; c < 3; ++c) {
            if (!on[c] || ea[c] || W->need[c]) continue;
            const double rr = v[c], sc2 = W->sig[c] * W->sig[c];
            if (isfinite(rr) && rr > 0.0 && rr * rr <= W->d2 * W->rref[c] * W->rref[c]) {
                W->need[c] = 1;
                W->sig_next[c] = pow2_scale(rr / sc2);
            }
        }
    W->any_need = need;
}

// x += e / sig in FP64 and e = 0 for the components about to be replaced (the
// scale of the iterations that made e); final: for every component not done
__global__ void __launch_bounds__(MB) k_m3_flush(M3Args a, int final) {
    const M3State *S = a.st;
    if (S->all_done || (!final && !S->any_need)) return;
    bool want[3];
    double isg[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        want[c] = !S->done[c] && (final || S->need[c]);
        isg[c] = 1.0 / S->sig[c];
    }
    for (int i = blockIdx.x * MB + threadIdx.x; i < a.n; i += gridDim.x * MB) {
        float4 e = a.e[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (!want[c]) continue;
            a.x[c][i] = fma((double)comp(e, c), isg[c], a.x[c][i]);
            comp(e, c) = 0.f;
        }
        a.e[i] = e;
    }
}

// statistics, and whether a component stalled; after_fp64: the FP64 solve that
// finished stalled components wrote its own, and the FP32 iterations are added
// to its counts
__global__ void k_m3_info(M3State *S, SolveInfo *info, int after_fp64) {
    for (int c = 0; c < 3; ++c) {
        if (after_fp64) {
            info->iters[c] += S->it[c];
            continue;
        }
        int st = S->status[c];
        if (st == DEV_OK && !S->done[c]) st = DEV_MAXITER;
        info->status[c] = st;
        info->iters[c] = S->it[c];
        info->res[c] = sqrt(S->rr64[c] / S->bb[c]);
    }
    info->refinements = S->upd[0] + S->upd[1] + S->upd[2];
    if (!after_fp64) {
        info->err = 0;
        S->stalled = S->status[0] == DEV_STALLED || S->status[1] == DEV_STALLED || S->status[2] == DEV_STALLED;
    }
}

}  // namespace

// Everything a captured solve bakes in: kernel arguments, grids, the scalars
// the set-up kernels take and the FP64 fallback's buffers.
struct M3Key {
    M3Args a;
    int g[8];
    int maxit, jacobi, sm_cap;
    double eps, d2, omega;
    long nnz;
    SolveInfo *info;
    const void *wbuf[10];
};

struct Bicg3Mixed::Impl {
    DevBuf<float4> r, rtd, p, v, s, t, e;
    DevBuf<float> dinv, sv32;
    DevBuf<double> r0;
    DevBuf<M3State> st;
    DevBuf<double> part;
    int n = 0;
    cudaGraphExec_t exec = nullptr;  // the whole solve, for streams that are not capturing
    long launches = 0;
    M3Key key{};
    ~Impl() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

Bicg3Mixed::Bicg3Mixed() : d_(new Impl) {}
Bicg3Mixed::~Bicg3Mixed() { delete d_; }

// Stream work of a solve, in pieces: the FP32 set-up; CH iterations; after the
// iterations, the unfinished components' flush and the statistics (which also
// record whether a component stalled); the FP64 solve of stalled components.
static void m3_setup(const M3Key &k, cudaStream_t st) {
    const M3Args &a = k.a;
    const int n = a.n;
    SYSU_CUDA(cudaMemsetAsync(a.st, 0, sizeof(M3State), st));
    // FP32 Jacobi weights and column-scaled matrix (FP64 would take a division per
    // row and a product per entry on the 1/64-rate FP64 pipe: 78 us of 2M rows)
    k_m3_dinv<<<(n + MB - 1) / MB, MB, 0, st>>>(a, (float)k.omega, k.jacobi);
    if (k.nnz > 0) k_m3_scale<<<(unsigned)((k.nnz + MB - 1) / MB), MB, 0, st>>>(a, k.nnz);
    k_m3_init<<<k.g[0], MB, 0, st>>>(a, k.maxit, k.eps, k.d2);
    k_m3_replace<<<k.g[1], MB, 0, st>>>(a, 1);
    g_launches += k.nnz > 0 ? 4 : 3;
    SYSU_CUDA(cudaGetLastError());
}

static void m3_chunk(const M3Key &k, cudaStream_t s) {
    const M3Args &a = k.a;
    const int *g = k.g;
    for (int it = 0; it < CH; ++it) {
        k_m3_dir<<<g[2], MB, 0, s>>>(a);
        k_m3_av<<<g[3], MB, 0, s>>>(a);
        k_m3_s<<<g[4], MB, 0, s>>>(a);
        k_m3_at<<<g[5], MB, 0, s>>>(a);
        k_m3_upd<<<g[6], MB, 0, s>>>(a);
        k_m3_flush<<<g[7], MB, 0, s>>>(a, 0);
        k_m3_replace<<<g[1], MB, 0, s>>>(a, 0);
    }
    g_launches += 7 * CH;
    SYSU_CUDA(cudaGetLastError());
}

static void m3_finish(const M3Key &k, cudaStream_t st) {
    // e of a component that the loop bound left unfinished (returns at once when
    // every component ended at a replacement)
    k_m3_flush<<<k.g[7], MB, 0, st>>>(k.a, 1);
    k_m3_info<<<1, 1, 0, st>>>(k.a.st, k.info, 0);
    g_launches += 2;
    SYSU_CUDA(cudaGetLastError());
}

static void m3_fp64(const M3Key &k, const SellDev &A, const double *val, const double *const *b, double *const *x,
                    const KrylovOpts &o, KrylovWork &w, cudaStream_t s) {
    // the FP64 batched solve from the current x (components already below eps take
    // no iteration), then the FP32 iterations added to its counts
    bicgstab_solve(A, val, 3, b, x, o, w, k.info, s);
    k_m3_info<<<1, 1, 0, s>>>(k.a.st, k.info, 1);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

// The solve as stream work on st (capturing): the set-up, the iterations as a
// graph WHILE node (the body's last kernel ends the loop once every component is
// done, or after a bound of bodies -- each iteration counts towards maxit and a
// component stalls after three replacements without progress, so the bound is
// never what ends a solve), the finish, and the FP64 solve of stalled
// components as an IF node.
static void m3_enqueue(const M3Key &k, const SellDev &A, const double *val, const double *const *b, double *const *x,
                       const KrylovOpts &o, KrylovWork &w, cudaStream_t st) {
    m3_setup(k, st);
    cudaStream_t side = graph_side_stream();
    const int bound = k.maxit / CH + 8;
    cudaGraphConditionalHandle loop = graph_cond_handle(st, 1);
    graph_cond_node(st, side, loop, cudaGraphCondTypeWhile, [&](cudaStream_t s) {
        m3_chunk(k, s);
        graph_loop_tail(loop, &k.a.st->all_done, &k.a.st->loops, bound, s);
    });
    m3_finish(k, st);
    cudaGraphConditionalHandle fb = graph_cond_handle(st, 0);
    graph_if_flag(fb, &k.a.st->stalled, st);
    graph_cond_node(st, side, fb, cudaGraphCondTypeIf,
                    [&](cudaStream_t s) { m3_fp64(k, A, val, b, x, o, w, s); });
}

void Bicg3Mixed::solve(const SellDev &A, const double *val, const double *const *b, double *const *x,
                       const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    const int n = A.n;
    if (n == 0) return;
    Impl &d = *d_;
    if (d.n < n) {
        d.r.alloc(n); d.rtd.alloc(n); d.p.alloc(n); d.v.alloc(n); d.s.alloc(n); d.t.alloc(n); d.e.alloc(n);
        d.dinv.alloc(n);
        d.r0.alloc((size_t)3 * n);
        d.n = n;
    }
    if (!d.st.size()) d.st.alloc(1);
    // each kernel on the blocks that fit at once (grid-stride row loops)
    static int res[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (!res[0]) {
        res[0] = coresident_blocks(k_m3_init, MB);
        res[1] = coresident_blocks(k_m3_replace, MB);
        res[2] = coresident_blocks(k_m3_dir, MB);
        res[3] = coresident_blocks(k_m3_av, MB);
        res[4] = coresident_blocks(k_m3_s, MB);
        res[5] = coresident_blocks(k_m3_at, MB);
        res[6] = coresident_blocks(k_m3_upd, MB);
        res[7] = coresident_blocks(k_m3_flush, MB);
    }
    M3Key k;
    std::memset(&k, 0, sizeof(k));  // padding too: the key is compared as bytes
    int gmax = 1;
    for (int j = 0; j < 8; ++j) {
        int nb = res[j];
        if (w.sm_cap > 0) nb = std::min(nb, w.sm_cap * std::max(1, res[j] / num_sms()));
        k.g[j] = std::max(1, std::min((n + MB - 1) / MB, nb));
        gmax = std::max(gmax, k.g[j]);
    }
    if (d.part.size() < (size_t)gmax * 9) d.part.alloc((size_t)gmax * 9);
    if (d.sv32.size() < (size_t)A.nnz) d.sv32.alloc(A.nnz);
    bicgstab_prepare(A, 3, w, st);  // the FP64 fallback's scratch, ahead of any capture
    M3Args &a = k.a;
    a.n = n;
    a.sl_ptr = A.sl_ptr.get();
    a.sl_w = A.sl_w.get();
    a.col = A.col.get();
    a.sv = d.sv32.get();
    a.val = val;
    a.dinv = d.dinv.get();
    a.r0 = d.r0.get();
    for (int c = 0; c < 3; ++c) {
        a.b[c] = b[c];
        a.x[c] = x[c];
    }
    a.r = d.r.get(); a.rtd = d.rtd.get(); a.p = d.p.get(); a.v = d.v.get(); a.s = d.s.get(); a.t = d.t.get();
    a.e = d.e.get();
    a.st = d.st.get();
    a.part = d.part.get();
    k.maxit = o.maxit;
    k.jacobi = o.jacobi ? 1 : 0;
    k.sm_cap = w.sm_cap;
    k.eps = o.eps;
    k.d2 = o.inner_tol * o.inner_tol;
    k.omega = o.omega;
    k.nnz = A.nnz;
    k.info = info;
    const void *wb[10] = {w.r.get(), w.rt.get(), w.p.get(), w.v.get(), w.s.get(),
                          w.t.get(), w.dinv.get(), w.partials.get(), w.sval.get(), w.barrier.get()};
    std::memcpy(k.wbuf, wb, sizeof(wb));
    if (stream_capturing(st)) {  // inside the caller's graph (the case batch)
        m3_enqueue(k, A, val, b, x, o, w, st);
        return;
    }
    if (!device_loop) {
        // host-driven form, for per-kernel profiling (profilers skip the kernels of
        // graphs with conditional nodes): the same kernels, CH iterations a captured
        // graph, the host reading the state after each
        k.maxit = -1 - k.maxit;  // a different cache entry from the device loop's
        if (!d.exec || std::memcmp(&k, &d.key, sizeof(M3Key)) != 0) {
            if (d.exec) cudaGraphExecDestroy(d.exec);
            d.exec = nullptr;
            const long before = g_launches.load();
            cudaGraph_t graph;
            SYSU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            m3_chunk(k, st);
            SYSU_CUDA(cudaStreamEndCapture(st, &graph));
            d.launches = g_launches.load() - before;
            g_launches -= d.launches;
            cudaError_t e = cudaGraphInstantiate(&d.exec, graph, 0);
            cudaGraphDestroy(graph);
            SYSU_CUDA(e);
            std::memcpy(&d.key, &k, sizeof(M3Key));
        }
        k.maxit = o.maxit;
        m3_setup(k, st);
        M3State h{};
        for (long it = 0; it < (long)o.maxit + 4L * CH; it += CH) {
            SYSU_CUDA(cudaGraphLaunch(d.exec, st));
            g_launches += d.launches;
            SYSU_CUDA(cudaMemcpyAsync(&h, d.st.get(), sizeof(M3State), cudaMemcpyDeviceToHost, st));
            SYSU_CUDA(cudaStreamSynchronize(st));
            if (h.all_done) break;
        }
        m3_finish(k, st);
        SYSU_CUDA(cudaMemcpyAsync(&h, d.st.get(), sizeof(M3State), cudaMemcpyDeviceToHost, st));
        SYSU_CUDA(cudaStreamSynchronize(st));
        if (h.stalled) m3_fp64(k, A, val, b, x, o, w, st);
        return;
    }
    if (!d.exec || std::memcmp(&k, &d.key, sizeof(M3Key)) != 0) {
        if (d.exec) cudaGraphExecDestroy(d.exec);
        d.exec = nullptr;
        const long before = g_launches.load();
        cudaGraph_t graph;
        SYSU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            m3_enqueue(k, A, val, b, x, o, w, st);
        } catch (...) {
            cudaGraph_t junk = nullptr;
            cudaStreamEndCapture(st, &junk);
            if (junk) cudaGraphDestroy(junk);
            throw;
        }
        SYSU_CUDA(cudaStreamEndCapture(st, &graph));
        d.launches = g_launches.load() - before;
        g_launches -= d.launches;
        cudaError_t e = cudaGraphInstantiate(&d.exec, graph, 0);
        cudaGraphDestroy(graph);
        SYSU_CUDA(e);
        std::memcpy(&d.key, &k, sizeof(M3Key));
    }
    SYSU_CUDA(cudaGraphLaunch(d.exec, st));
    g_launches += d.launches;
}

}  // namespace sysu
