// Jacobi-preconditioned CG on SELL-32 matrices: FP64, and FP32 recurrences
// with reliable FP64 updates.  Replaces LASPack's CGIter as the reference calls
// it for the pressure correction and the solid conduction equation
// (navier_pressure.cpp:29, HeatConductionSolver.cpp:90 through SolveLinearEqu,
// tools.cpp:56-64): same recurrences (Barrett et al., "Templates", Fig. 2.5),
// same stopping test ||b - A x||_2 / ||b||_2 < eps, same iteration cap.
//
// One solve = one cooperative launch of a persistent kernel, one 1024-thread
// CTA per SM: 31 consumer warps and one producer warp.  Each CTA owns a
// contiguous range of slices (32-row groups of the SELL matrix), cut into
// tiles of TS = 31 slices -- one row per consumer thread.  An iteration is
// three phases over the CTA's tiles:
//   U  p = z + beta p                    reads z, p        writes p
//   S  q = A p, p.q                      reads val, col    writes q   (gathers p)
//   X  x += alpha p, r -= alpha q, z = M^-1 r, r.r, r.z
//                                        reads p q x r dinv  writes x, r, z
// separated by a grid barrier (U -> S) and two deterministic grid reductions.
// Every operand a phase streams (everything but the gathered p) is moved into
// shared memory by bulk asynchronous copies (cp.async.bulk, the TMA engine's
// 1-D form) through a ring of D slots, so the DRAM stream runs ahead of the
// arithmetic: while the consumers compute tile j, tiles j+1 .. j+D-1 are in
// flight, also across phase boundaries and grid barriers.  The matrix is
// copied with an L2 evict-first policy so the vectors (about 100 MB at 2M rows
// in FP64) stay in the 126 MB L2 between phases.
//
// Ring protocol (per CTA): job j = (phase, tile) in consumption order lives in
// slot j % D.  A slot's "full" mbarrier completes when its bytes land, its
// "empty" mbarrier when all consumer warps are done with it.  Lane 0 of the
// producer warp issues jobs in order as soon as the previous user of the slot
// has been released, within a budget of released jobs.  Tiles of a phase that
// read vectors the previous phase wrote are released at that phase's end,
// after every thread's fence.proxy.async (which orders its plain stores before
// later bulk-copy reads) and a block barrier; the matrix tiles of S are
// released with U.  In its loop over phase P the producer blocks (bounded)
// only for P's own tiles and issues later ones only when a slot is free, so it
// always reaches the block barrier at the end of P.  Every wait is bounded; a
// CTA drains its copies before it leaves.
#include <climits>

#include "bulk.cuh"
#include "krylov_dev.cuh"

namespace sysu {
namespace {

constexpr int CG_CONSUMERS = KBC / 32 - 1;          // consumer warps; warp 31 produces
constexpr int CG_PRODUCER = KBC / 32 - 1;
constexpr int CG_MAX_TS = CG_CONSUMERS;             // 31 slices = 992 rows per tile
constexpr unsigned CG_SMEM_BUDGET = 200 * 1024;     // dynamic shared memory for the ring

enum CgPhase { PH_U = 0, PH_S = 1, PH_X = 2 };

// Launch plan: slices per tile, ring depth, slot size.
struct CgPlan {
    int ts = CG_MAX_TS;
    int depth = 2;
    unsigned slot = 0;     // bytes per slot (multiple of 128)
    int direct = 0;        // 1: S tiles read val/col from global (rows too long for a slot)
    unsigned smem = 0;     // dynamic shared memory bytes
};

struct CgPipeArgs {
    SellView A;             // FP64 values
    const float *val32;     // FP32 values (mixed)
    const double *b;
    double *x;
    double *r, *z, *p, *q;  // FP64 solve
    const double *dinv;
    float *r32, *z32, *p32, *q32, *e32;  // mixed solve
    const float *dinv32;
    double *partials;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit;
    double eps, inner_tol;
    unsigned long long *ts;
    CgPlan plan;
};

__shared__ uint64_t g_full[CopyRing::DMAX];
__shared__ uint64_t g_empty[CopyRing::DMAX];
__shared__ int g_fail;
extern __shared__ __align__(128) unsigned char g_slots[];

// The CTA's share of the matrix and the geometry of its tiles.
struct Part {
    int n, sb, se, nt, ts;
    __device__ void tile(int t, int &s0, int &s1, int &r0, int &nr) const {
        s0 = sb + t * ts;
        s1 = min(s0 + ts, se);
        r0 = s0 * 32;
        nr = min(s1 * 32, n) - r0;
    }
};

__device__ __forceinline__ Part make_part(int n, int nslices, int ts) {
    Part P;
    P.n = n;
    P.ts = ts;
    P.sb = (int)((long long)nslices * blockIdx.x / gridDim.x);
    P.se = (int)((long long)nslices * (blockIdx.x + 1) / gridDim.x);
    P.nt = (P.se - P.sb + ts - 1) / ts;
    return P;
}

__device__ __forceinline__ int fail_flag() { return *reinterpret_cast<volatile int *>(&g_fail); }
__device__ __forceinline__ void set_fail(int *err) {
    *reinterpret_cast<volatile int *>(&g_fail) = 1;
    atomicExch(err, (int)DEV_BARRIER_TIMEOUT);
}

// Ring state.  The consumer side (Ring, in registers) is uniform across the
// consumer warps; the producer side (Producer, in shared memory) is touched by
// the producer lane only.  A CTA runs its ring at depth min(D, nt).
struct Ring {
    int depth;
    unsigned slot;
    int cslot;          // slot of the next job to consume
    unsigned cpar;      // its full-barrier phase parity
};
struct Producer {
    long long issued;   // jobs issued
    long long allowed;  // jobs released so far (issue limit)
    int nt;
    int islot;          // slot of the next job to issue
    unsigned ipar;      // its round parity
    int iph, itile;     // phase and tile of the next job to issue
    int primed;         // jobs issued so far, saturating at depth
};
__shared__ Producer g_prod;

// First matrix entry of every tile of the CTA (entry offsets of the S tiles),
// so that issuing a tile needs no global load.
constexpr int CG_TILE_TABLE = 1024;
__shared__ int g_tile_e[CG_TILE_TABLE + 1];

__device__ __forceinline__ int tile_entry(const Part &P, const int *sl_ptr, int t) {
    return t <= CG_TILE_TABLE ? g_tile_e[t] : __ldg(sl_ptr + min(P.sb + t * P.ts, P.se));
}


__device__ __forceinline__ bool is_producer() { return (threadIdx.x >> 5) == CG_PRODUCER; }
__device__ __forceinline__ bool is_producer_lane() { return threadIdx.x == CG_PRODUCER * 32; }

__device__ __forceinline__ unsigned char *cslot_ptr(const Ring &R) { return g_slots + (size_t)R.cslot * R.slot; }

// Producer warp (all 32 lanes, converged): issue jobs in order within the
// budget; wait (bounded) for a slot only for jobs before `must_end`, stop at
// the first busy slot otherwise.  Lane 0 issues the copies and takes the
// barrier decisions, broadcast to the warp, so the warp never diverges across
// the block barriers and warp collectives that follow.  The state is worked on
// in registers (the copy instructions clobber memory).
template <class Issue>
__device__ __forceinline__ bool produce(const Ring &R, long long must_end, Issue &&issue) {
    Producer &Q = g_prod;
    const bool lead = (threadIdx.x & 31) == 0;
    long long issued = Q.issued;
    const long long allowed = Q.allowed;
    if (issued >= allowed) return true;
    const int nt = Q.nt, depth = R.depth;
    int islot = Q.islot, iph = Q.iph, itile = Q.itile, primed = Q.primed;
    unsigned ipar = Q.ipar;
    const uint64_t pol_stream = l2_policy_evict_first();
    const uint64_t pol_keep = l2_policy_evict_last();
    bool ok = true;
    while (issued < allowed) {
        if (primed == depth) {  // the slot's previous job must be released by all consumers
            int free_slot = lead ? (int)mbar_test_wait(&g_empty[islot], ipar ^ 1u) : 0;
            free_slot = __shfl_sync(FULL_MASK, free_slot, 0);
            if (!free_slot) {
                if (issued >= must_end) break;  // never wait for a look-ahead tile
                int got = lead ? (int)mbar_wait(&g_empty[islot], ipar ^ 1u) : 0;
                if (!__shfl_sync(FULL_MASK, got, 0)) { ok = false; break; }
            }
        } else {
            ++primed;
        }
        if (lead) issue(iph, itile, g_slots + (size_t)islot * R.slot, &g_full[islot], pol_stream, pol_keep);
        __syncwarp();
        if (++islot == depth) { islot = 0; ipar ^= 1u; }
        if (++itile == nt) { itile = 0; if (++iph == 3) iph = 0; }
        ++issued;
    }
    __syncwarp();
    if (lead) {
        Q.issued = issued;
        Q.islot = islot;
        Q.ipar = ipar;
        Q.iph = iph;
        Q.itile = itile;
        Q.primed = primed;
    }
    __syncwarp();
    return ok;
}

// The producer warp's part of a phase: issue the phase's remaining tiles
// (jobs before must_end) and whatever later tiles fit.
template <class Issue>
__device__ __forceinline__ void producer_phase(const Ring &R, long long must_end, Issue &&issue, int *err) {
    if (!is_producer()) return;
    bool ok = __all_sync(FULL_MASK, !fail_flag()) ? produce(R, must_end, issue) : true;
    if (!ok && (threadIdx.x & 31) == 0) set_fail(err);
}

// Consumer warps: wait until the next job has landed.  The outcome is uniform
// per warp; false after a timed-out wait (recorded in g_fail and *err).
__device__ __forceinline__ bool acquire(const Ring &R, int *err) {
    bool ok = !__any_sync(FULL_MASK, fail_flag() != 0);
    if (ok) ok = mbar_wait(&g_full[R.cslot], R.cpar);
    ok = __all_sync(FULL_MASK, ok);
    if (!ok && (threadIdx.x & 31) == 0) set_fail(err);
    return ok;
}

// Consumer warps, after their last read of the slot: release it.
__device__ __forceinline__ void release(Ring &R) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&g_empty[R.cslot])) : "memory");
    if (++R.cslot == R.depth) { R.cslot = 0; R.cpar ^= 1u; }
}

// Producer lane at exit: wait (bounded) for the last copy issued into each
// slot (a slot's copies complete in order), so none is in flight when the CTA
// leaves, whether or not its tile was consumed.
__device__ __forceinline__ void drain(const Ring &R) {
    if (!is_producer_lane()) return;
    long long issued = g_prod.issued;
    for (int s = 0; s < R.depth; ++s) {
        long long last = issued - 1 - ((issued - 1 - s) % R.depth + R.depth) % R.depth;
        if (last < 0) continue;
        if (!mbar_wait(&g_full[s], (unsigned)((last / R.depth) & 1))) break;
    }
}

__device__ __forceinline__ void ring_init(Ring &R, const CgPlan &pl, const Part &P, const int *sl_ptr,
                                          long long allowed) {
    const int nt = P.nt;
    for (int t = threadIdx.x; t <= min(nt, CG_TILE_TABLE); t += blockDim.x)
        g_tile_e[t] = __ldg(sl_ptr + min(P.sb + t * P.ts, P.se));
    R.depth = max(1, min(pl.depth, nt));
    R.slot = pl.slot;
    R.cslot = 0;
    R.cpar = 0u;
    if (threadIdx.x == 0) {
        Producer &Q = g_prod;
        Q.issued = 0;
        Q.allowed = allowed;
        Q.nt = nt;
        Q.islot = 0;
        Q.ipar = 0u;
        Q.iph = Q.itile = 0;
        Q.primed = 0;
        for (int k = 0; k < R.depth; ++k) {
            mbar_init(&g_full[k], 1);
            mbar_init(&g_empty[k], CG_CONSUMERS);
        }
        g_fail = 0;
        mbar_init_fence();
    }
    __syncthreads();
}

// Every thread at the end of a phase: publish this phase's plain stores to the
// async proxy (one fence per thread per phase), block barrier, then the
// producer releases `more` further jobs -- tiles of the next phase, whose
// copies read those stores -- and issues what fits, so they land while the
// CTA waits in the grid barrier that follows.
template <class Issue>
__device__ __forceinline__ void phase_end(const Ring &R, int more, Issue &&issue, int *err) {
    fence_proxy_async_global();
    __syncthreads();
    if (is_producer() && __all_sync(FULL_MASK, !fail_flag())) {
        if ((threadIdx.x & 31) == 0) g_prod.allowed += more;
        __syncwarp();
        if (!produce(R, 0, issue) && (threadIdx.x & 31) == 0) set_fail(err);
    }
}

// Loop state code from the squared residual: 1 converged (||r||^2 < thr,
// thr = eps^2 ||b||^2, the stopping test ||r|| / ||b|| < eps without a square
// root or division per iteration), 2 not finite, 0 go on.
__device__ __forceinline__ double stop_code(double rr, double thr) {
    return rr < thr ? 1.0 : (isfinite(rr) ? 0.0 : 2.0);
}

// One SELL row of a tile: the column indices of up to 8 entries, then their
// gathers, then the FMAs.
template <class V, class X, class Acc>
__device__ __forceinline__ Acc tile_row_dot(const V *vs, const int *cs, int e, int w, const X *__restrict__ x,
                                            X &diag) {
    if (w <= 0) {
        diag = (X)0;
        return (Acc)0;
    }
    X xv[8];
    int c[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) c[k] = cs[e + 32 * k];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < w) xv[k] = x[c[k]];
    Acc acc = (Acc)vs[e] * (Acc)xv[0];
#pragma unroll
    for (int k = 1; k < 8; ++k)
        if (k < w) acc = fma((Acc)vs[e + 32 * k], (Acc)xv[k], acc);
    for (int k = 8; k < w; ++k) acc = fma((Acc)vs[e + 32 * k], (Acc)x[cs[e + 32 * k]], acc);
    diag = xv[0];
    return acc;
}

// ---------------------------------------------------------------------------
// FP64
__global__ void __launch_bounds__(KBC, 1) k_cg_pipe(CgPipeArgs a) {
    const int n = a.A.n;
    const int tid = threadIdx.x;
    const bool prod = is_producer();
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const Part P = make_part(n, a.A.nslices, a.plan.ts);
    const int nt = P.nt;
    const unsigned VS = (unsigned)P.ts * 32 * sizeof(double);  // vector stride in a slot
    const int R0 = P.sb * 32, R1 = min(P.se * 32, n);
    Ring R;
    ring_init(R, a.plan, P, a.A.sl_ptr, 2LL * nt);  // U and S tiles of the first iteration

    // r = b - A x, z = M^-1 r; ||b||^2, ||r||^2, r.z
    double v3[3] = {0.0, 0.0, 0.0};
    for (int i = R0 + tid; i < R1; i += KBC) {
        double bi = a.b[i];
        double ri = bi - row_dot(a.A, i, a.x);
        double zi = a.dinv[i] * ri;
        a.r[i] = ri;
        a.z[i] = zi;
        v3[0] += bi * bi;
        v3[1] += ri * ri;
        v3[2] += ri * zi;
    }
    fence_proxy_async_global();
    if (!grid_sum_t0<3>(v3, rc, a.gb, err)) { drain(R); return; }
    // thread-0 scalar state, kept in shared memory (no registers in the other threads)
    __shared__ double s_state[4];
    double &bb = s_state[0], &rr = s_state[1], &rho = s_state[2], &thr = s_state[3];
    if (tid == 0) {
        bb = v3[0] == 0.0 ? 1.0 : v3[0];
        thr = a.eps * a.eps * bb;
        rr = v3[1];
        rho = v3[2];
        g_bc[0] = stop_code(rr, thr);
        g_bc[1] = 0.0;
    }
    __syncthreads();

    auto issue = [&](int ph, int t, unsigned char *dst, uint64_t *bar, uint64_t pol_stream, uint64_t pol_keep) {
        int s0, s1, r0, nr;
        P.tile(t, s0, s1, r0, nr);
        unsigned vb = (unsigned)(nr * 8) & ~15u;
        if (ph == PH_S) {
            if (a.plan.direct) { mbar_arrive_expect_tx(bar, 0); return; }
            long e0 = tile_entry(P, a.A.sl_ptr, t), e1 = tile_entry(P, a.A.sl_ptr, t + 1);
            unsigned bv = (unsigned)((e1 - e0) * 8), bc = (unsigned)((e1 - e0) * 4);
            mbar_arrive_expect_tx(bar, bv + bc);
            if (bv) {
                bulk_g2s(dst, a.A.val + e0, bv, bar, pol_stream);
                bulk_g2s(dst + bv, a.A.col + e0, bc, bar, pol_stream);
            }
        } else if (ph == PH_U) {
            mbar_arrive_expect_tx(bar, 2 * vb);
            if (vb) {
                bulk_g2s(dst, a.z + r0, vb, bar, pol_keep);
                bulk_g2s(dst + VS, a.p + r0, vb, bar, pol_keep);
            }
        } else {
            mbar_arrive_expect_tx(bar, 5 * vb);
            if (vb) {
                bulk_g2s(dst, a.p + r0, vb, bar, pol_keep);
                bulk_g2s(dst + VS, a.q + r0, vb, bar, pol_keep);
                bulk_g2s(dst + 2 * VS, a.x + r0, vb, bar, pol_keep);
                bulk_g2s(dst + 3 * VS, a.r + r0, vb, bar, pol_keep);
                bulk_g2s(dst + 4 * VS, a.dinv + r0, vb, bar, pol_keep);
            }
        }
    };

    long long base = 0;  // job index of the current phase's first tile
    int it = 0, status = DEV_OK;
    for (;;) {
        double code = g_bc[0], beta = g_bc[1];
        __syncthreads();
        if (code == 1.0 || it >= a.maxit) break;
        if (code == 2.0) { status = DEV_NONFINITE; break; }
        ++it;
        stamp(a.ts, it, 0);
        // U
        if (prod) {
            producer_phase(R, base + nt, issue, err);
        } else {
            for (int t = 0; t < nt; ++t) {
                if (!acquire(R, err)) break;
                const double *sp = reinterpret_cast<const double *>(cslot_ptr(R));
                int s0, s1, r0, nr;
                P.tile(t, s0, s1, r0, nr);
                if (tid < nr) {
                    int i = r0 + tid;
                    bool tma = tid < (nr & ~1);
                    double zi = tma ? sp[tid] : a.z[i];
                    double pi = tma ? sp[VS / 8 + tid] : a.p[i];
                    a.p[i] = (it == 1) ? zi : fma(beta, pi, zi);
                }
                release(R);
            }
        }
        base += nt;
        if (!grid_sync(a.gb, err) || fail_flag()) break;
        stamp(a.ts, it, 1);
        // S
        double v1[1] = {0.0};
        if (prod) {
            producer_phase(R, base + nt, issue, err);
        } else {
            for (int t = 0; t < nt; ++t) {
                if (!acquire(R, err)) break;
                int s0, s1, r0, nr;
                P.tile(t, s0, s1, r0, nr);
                if (tid < nr) {
                    int s = s0 + (tid >> 5);
                    int e0 = tile_entry(P, a.A.sl_ptr, t), e1 = tile_entry(P, a.A.sl_ptr, t + 1);
                    int es = __ldg(a.A.sl_ptr + s) - e0 + (tid & 31);
                    int w = __ldg(a.A.sl_w + s);
                    const double *vs;
                    const int *cs;
                    if (a.plan.direct) {
                        vs = a.A.val + e0;
                        cs = a.A.col + e0;
                    } else {
                        vs = reinterpret_cast<const double *>(cslot_ptr(R));
                        cs = reinterpret_cast<const int *>(cslot_ptr(R) + (size_t)(e1 - e0) * 8);
                    }
                    double pi;
                    double qi = tile_row_dot<double, double, double>(vs, cs, es, w, a.p, pi);
                    a.q[r0 + tid] = qi;
                    v1[0] = fma(pi, qi, v1[0]);
                }
                release(R);
            }
        }
        base += nt;
        phase_end(R, nt, issue, err);  // X tiles read p and q
        if (!grid_sum_t0<1>(v1, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, it, 2);
        if (tid == 0) {
            g_bc[2] = v1[0] == 0.0 ? 0.0 : rho / v1[0];
            g_bc[3] = v1[0] == 0.0 ? 1.0 : 0.0;
        }
        __syncthreads();
        double alpha = g_bc[2];
        if (g_bc[3] != 0.0) { status = DEV_BREAKDOWN; break; }
        // X
        double v2[2] = {0.0, 0.0};
        if (prod) {
            producer_phase(R, base + nt, issue, err);
        } else {
            for (int t = 0; t < nt; ++t) {
                if (!acquire(R, err)) break;
                const double *sp = reinterpret_cast<const double *>(cslot_ptr(R));
                int s0, s1, r0, nr;
                P.tile(t, s0, s1, r0, nr);
                if (tid < nr) {
                    int i = r0 + tid;
                    const unsigned V = VS / 8;
                    double pi, qi, xi, ri, di;
                    if (tid < (nr & ~1)) {
                        pi = sp[tid]; qi = sp[V + tid]; xi = sp[2 * V + tid]; ri = sp[3 * V + tid]; di = sp[4 * V + tid];
                    } else {
                        pi = a.p[i]; qi = a.q[i]; xi = a.x[i]; ri = a.r[i]; di = a.dinv[i];
                    }
                    xi = fma(alpha, pi, xi);
                    ri = fma(-alpha, qi, ri);
                    double zi = di * ri;
                    a.x[i] = xi;
                    a.r[i] = ri;
                    a.z[i] = zi;
                    v2[0] = fma(ri, ri, v2[0]);
                    v2[1] = fma(ri, zi, v2[1]);
                }
                release(R);
            }
        }
        base += nt;
        phase_end(R, 2 * nt, issue, err);  // next U tiles read z and p; S tiles
        if (!grid_sum_t0<2>(v2, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, it, 3);
        if (tid == 0) {
            rr = v2[0];
            g_bc[0] = stop_code(rr, thr);
            g_bc[1] = v2[1] / rho;
            rho = v2[1];
        }
        __syncthreads();
    }
    drain(R);
    if (blockIdx.x == 0 && tid == 0) {
        double res = sqrt(rr) / sqrt(bb);
        if (status == DEV_OK && !(rr < thr)) status = isfinite(rr) ? DEV_MAXITER : DEV_NONFINITE;
        a.info->status[0] = status;
        a.info->iters[0] = it;
        a.info->res[0] = res;
    }
}

// ---------------------------------------------------------------------------
// Mixed precision: the recurrences (p, q, r, z and the correction e) run in
// FP32, with reliable updates (Sleijpen & van der Vorst, "Reliable updated
// residuals in hybrid Bi-CG methods", Computing 56, 1996): once the FP32
// residual has fallen by inner_tol since the last update, e is added to the
// FP64 solution, e is zeroed, the FP64 residual b - A x replaces the FP32 one
// and the search direction is kept, so the Krylov process is not restarted.
// Convergence is decided on that FP64 residual only.  Per-thread partial dot
// products run in FP32 over the thread's rows; FP64 across threads.
__global__ void __launch_bounds__(KBC, 1) k_cg_mixed_pipe(CgPipeArgs a) {
    const int n = a.A.n;
    const int tid = threadIdx.x;
    const bool prod = is_producer();
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const Part P = make_part(n, a.A.nslices, a.plan.ts);
    const int nt = P.nt;
    const unsigned VS = (unsigned)P.ts * 32 * sizeof(float);
    const int R0 = P.sb * 32, R1 = min(P.se * 32, n);
    const float *__restrict__ dinv = a.dinv32;
    Ring R;
    ring_init(R, a.plan, P, a.A.sl_ptr, 0);

    // FP64 residual of the initial guess and its FP32 copy
    double v3[3] = {0.0, 0.0, 0.0};
    float f2 = 0.f;
    for (int i = R0 + tid; i < R1; i += KBC) {
        double bi = a.b[i];
        double ri = bi - row_dot(a.A, i, a.x);
        float rf = (float)ri, zf = dinv[i] * rf;
        a.r32[i] = rf;
        a.z32[i] = zf;
        a.e32[i] = 0.f;
        v3[0] += bi * bi;
        v3[1] += ri * ri;
        f2 = fmaf(rf, zf, f2);
    }
    v3[2] = (double)f2;
    fence_proxy_async_global();
    if (!grid_sum_t0<3>(v3, rc, a.gb, err)) { drain(R); return; }
    // thread-0 scalar state, kept in shared memory (no registers in the other threads);
    // rr_ref: FP64 ||b - A x||^2 at the last reliable update
    __shared__ double s_state[4];
    double &bb = s_state[0], &thr = s_state[1], &rho = s_state[2], &rr_ref = s_state[3];
    if (tid == 0) {
        bb = v3[0] == 0.0 ? 1.0 : v3[0];
        thr = a.eps * a.eps * bb;
        rr_ref = v3[1];
        rho = v3[2];
        g_bc[0] = stop_code(rr_ref, thr);
        g_bc[1] = 0.0;
    }
    __syncthreads();

    auto issue = [&](int ph, int t, unsigned char *dst, uint64_t *bar, uint64_t pol_stream, uint64_t pol_keep) {
        int s0, s1, r0, nr;
        P.tile(t, s0, s1, r0, nr);
        unsigned vb = (unsigned)(nr * 4) & ~15u;
        if (ph == PH_S) {
            if (a.plan.direct) { mbar_arrive_expect_tx(bar, 0); return; }
            long e0 = tile_entry(P, a.A.sl_ptr, t), e1 = tile_entry(P, a.A.sl_ptr, t + 1);
            unsigned bv = (unsigned)((e1 - e0) * 4);
            mbar_arrive_expect_tx(bar, 2 * bv);
            if (bv) {
                bulk_g2s(dst, a.val32 + e0, bv, bar, pol_stream);
                bulk_g2s(dst + bv, a.A.col + e0, bv, bar, pol_stream);
            }
        } else if (ph == PH_U) {
            mbar_arrive_expect_tx(bar, 2 * vb);
            if (vb) {
                bulk_g2s(dst, a.z32 + r0, vb, bar, pol_keep);
                bulk_g2s(dst + VS, a.p32 + r0, vb, bar, pol_keep);
            }
        } else {
            mbar_arrive_expect_tx(bar, 5 * vb);
            if (vb) {
                bulk_g2s(dst, a.p32 + r0, vb, bar, pol_keep);
                bulk_g2s(dst + VS, a.q32 + r0, vb, bar, pol_keep);
                bulk_g2s(dst + 2 * VS, a.e32 + r0, vb, bar, pol_keep);
                bulk_g2s(dst + 3 * VS, a.r32 + r0, vb, bar, pol_keep);
                bulk_g2s(dst + 4 * VS, dinv + r0, vb, bar, pol_keep);
            }
        }
    };

    long long base = 0;  // job index of the current phase's first tile
    int total = 0, nupd = 0, status = DEV_OK;
    for (;;) {
        double code = g_bc[0];  // from the FP64 residual of the last update
        float beta = (float)g_bc[1];
        __syncthreads();
        if (code == 1.0 || total >= a.maxit) break;
        if (code == 2.0) { status = DEV_NONFINITE; break; }
        ++total;
        stamp(a.ts, total, 0);
        // U tiles read z, which a reliable update rewrites: they are released
        // only here, with this iteration's S tiles (X tiles at the end of S)
        if (is_producer_lane()) g_prod.allowed = base + 2LL * nt;
        __syncwarp();
        if (prod) {
            producer_phase(R, base + nt, issue, err);
        } else {
            for (int t = 0; t < nt; ++t) {
                if (!acquire(R, err)) break;
                const float *sp = reinterpret_cast<const float *>(cslot_ptr(R));
                int s0, s1, r0, nr;
                P.tile(t, s0, s1, r0, nr);
                if (tid < nr) {
                    int i = r0 + tid;
                    bool tma = tid < (nr & ~3);
                    float zi = tma ? sp[tid] : a.z32[i];
                    float pi = tma ? sp[VS / 4 + tid] : a.p32[i];
                    a.p32[i] = (total == 1) ? zi : fmaf(beta, pi, zi);
                }
                release(R);
            }
        }
        base += nt;
        if (!grid_sync(a.gb, err) || fail_flag()) break;
        stamp(a.ts, total, 1);
        float g0 = 0.f;
        if (prod) {
            producer_phase(R, base + nt, issue, err);
        } else {
            for (int t = 0; t < nt; ++t) {
                if (!acquire(R, err)) break;
                int s0, s1, r0, nr;
                P.tile(t, s0, s1, r0, nr);
                if (tid < nr) {
                    int s = s0 + (tid >> 5);
                    int e0 = tile_entry(P, a.A.sl_ptr, t), e1 = tile_entry(P, a.A.sl_ptr, t + 1);
                    int es = __ldg(a.A.sl_ptr + s) - e0 + (tid & 31);
                    int w = __ldg(a.A.sl_w + s);
                    const float *vs;
                    const int *cs;
                    if (a.plan.direct) {
                        vs = a.val32 + e0;
                        cs = a.A.col + e0;
                    } else {
                        vs = reinterpret_cast<const float *>(cslot_ptr(R));
                        cs = reinterpret_cast<const int *>(cslot_ptr(R) + (size_t)(e1 - e0) * 4);
                    }
                    float pi;
                    float qi = tile_row_dot<float, float, float>(vs, cs, es, w, a.p32, pi);
                    a.q32[r0 + tid] = qi;
                    g0 = fmaf(pi, qi, g0);
                }
                release(R);
            }
        }
        base += nt;
        phase_end(R, nt, issue, err);  // X tiles read p and q
        double v1[1] = {(double)g0};
        if (!grid_sum_t0<1>(v1, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, total, 2);
        if (tid == 0) {
            g_bc[2] = v1[0] == 0.0 ? 0.0 : rho / v1[0];
            g_bc[3] = v1[0] == 0.0 ? 1.0 : 0.0;
        }
        __syncthreads();
        float alpha = (float)g_bc[2];
        if (g_bc[3] != 0.0) { status = DEV_BREAKDOWN; break; }
        float h0 = 0.f, h1 = 0.f;
        if (prod) {
            producer_phase(R, base + nt, issue, err);
        } else {
            for (int t = 0; t < nt; ++t) {
                if (!acquire(R, err)) break;
                const float *sp = reinterpret_cast<const float *>(cslot_ptr(R));
                int s0, s1, r0, nr;
                P.tile(t, s0, s1, r0, nr);
                if (tid < nr) {
                    int i = r0 + tid;
                    const unsigned V = VS / 4;
                    float pi, qi, ei, ri, di;
                    if (tid < (nr & ~3)) {
                        pi = sp[tid]; qi = sp[V + tid]; ei = sp[2 * V + tid]; ri = sp[3 * V + tid]; di = sp[4 * V + tid];
                    } else {
                        pi = a.p32[i]; qi = a.q32[i]; ei = a.e32[i]; ri = a.r32[i]; di = dinv[i];
                    }
                    ei = fmaf(alpha, pi, ei);
                    ri = fmaf(-alpha, qi, ri);
                    float zi = di * ri;
                    a.e32[i] = ei;
                    a.r32[i] = ri;
                    a.z32[i] = zi;
                    h0 = fmaf(ri, ri, h0);
                    h1 = fmaf(ri, zi, h1);
                }
                release(R);
            }
        }
        base += nt;
        phase_end(R, 0, issue, err);  // next U tiles read z and p
        double w2[2] = {(double)h0, (double)h1};
        if (!grid_sum_t0<2>(w2, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, total, 3);
        if (tid == 0) {
            // reliable update once the FP32 residual fell by inner_tol since the
            // last one, when it looks converged, or at the iteration cap
            const double d2 = a.inner_tol * a.inner_tol;
            bool upd = w2[0] <= d2 * rr_ref || w2[0] <= thr || total >= a.maxit || !(w2[0] == w2[0]);
            if (!upd) {
                g_bc[1] = w2[1] / rho;
                rho = w2[1];
            }
            g_bc[4] = upd ? 1.0 : 0.0;
        }
        __syncthreads();
        if (g_bc[4] != 0.0) {
            for (int i = R0 + tid; i < R1; i += KBC) {
                a.x[i] += (double)a.e32[i];
                a.e32[i] = 0.f;
            }
            if (!grid_sync(a.gb, err)) break;
            double u[2] = {0.0, 0.0};
            float fz = 0.f;
            for (int i = R0 + tid; i < R1; i += KBC) {
                double ri = a.b[i] - row_dot(a.A, i, a.x);
                float rf = (float)ri, zf = dinv[i] * rf;
                a.r32[i] = rf;
                a.z32[i] = zf;
                u[0] += ri * ri;
                fz = fmaf(rf, zf, fz);
            }
            u[1] = (double)fz;
            fence_proxy_async_global();
            if (!grid_sum_t0<2>(u, rc, a.gb, err)) break;
            if (tid == 0) {
                rr_ref = u[0];
                g_bc[0] = stop_code(rr_ref, thr);
                g_bc[1] = u[1] / rho;  // keep the direction: beta from the replaced residual
                rho = u[1];
                ++nupd;
            }
            __syncthreads();
        }
    }
    drain(R);
    if (status == DEV_BREAKDOWN)  // keep the correction gathered so far
        for (int i = R0 + tid; i < R1; i += KBC) a.x[i] += (double)a.e32[i];
    if (blockIdx.x == 0 && tid == 0) {
        double res = sqrt(rr_ref) / sqrt(bb);
        if (status == DEV_OK && !(rr_ref < thr)) status = isfinite(rr_ref) ? DEV_MAXITER : DEV_NONFINITE;
        a.info->status[0] = status;
        a.info->iters[0] = total;
        a.info->res[0] = res;
        a.info->refinements = nupd;
    }
}

__global__ void k_dinv32(SellView A, double omega, float *dinv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    dinv[i] = (float)(omega / A.val[A.sl_ptr[i >> 5] + (i & 31)]);
}

// Tile size and ring depth for a matrix whose widest slice has wmax entries
// per row; ebytes = bytes per matrix value.
CgPlan plan_cg(int wmax, int ebytes) {
    CgPlan pl;
    auto round128 = [](unsigned b) { return (b + 127u) & ~127u; };
    for (int ts = CG_MAX_TS; ts >= 1; ts /= 2) {
        unsigned vec = 5u * ts * 32 * ebytes;
        unsigned mat = (unsigned)ts * 32 * (unsigned)wmax * (unsigned)(ebytes + 4);
        unsigned slot = round128(std::max(vec, mat));
        int depth = (int)std::min<unsigned>(CopyRing::DMAX, CG_SMEM_BUDGET / slot);
        if (depth >= 2) {
            pl.ts = ts;
            pl.depth = depth;
            pl.slot = slot;
            pl.smem = slot * depth;
            return pl;
        }
    }
    // rows too long for a slot: S tiles read the matrix from global memory
    pl.ts = CG_MAX_TS;
    pl.direct = 1;
    pl.slot = round128(5u * CG_MAX_TS * 32 * ebytes);
    pl.depth = (int)std::min<unsigned>(CopyRing::DMAX, CG_SMEM_BUDGET / pl.slot);
    pl.smem = pl.slot * pl.depth;
    return pl;
}

template <class K>
int cg_max_blocks(K kernel) {
    SYSU_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CG_SMEM_BUDGET));
    int per_sm = 0;
    SYSU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, KBC, CG_SMEM_BUDGET));
    if (per_sm < 1) throw CaseError{"persistent CG kernel cannot be resident"};
    return per_sm * num_sms();
}

int cg_grid(const SellDev &A, const CgPlan &pl, int maxb) {
    int tiles = (A.nslices + pl.ts - 1) / pl.ts;
    return std::max(1, std::min(tiles, maxb));
}

}  // namespace

void cg_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
              const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = cg_max_blocks(k_cg_pipe);
    w.ensure(n, 1, maxb, st);
    check_aligned16({x, val, A.col.get(), w.r.get(), w.s.get(), w.p.get(), w.v.get(), w.dinv.get()});
    SellView V = view(A, val);
    { k_jacobi_dinv<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, o.jacobi ? 1 : 0, w.dinv.get()); ++::sysu::g_launches; }
    if (x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    CgPipeArgs a{};
    a.A = V;
    a.b = b;
    a.x = x;
    a.r = w.r.get();
    a.z = w.s.get();
    a.p = w.p.get();
    a.q = w.v.get();
    a.dinv = w.dinv.get();
    a.partials = w.partials.get();
    a.gb = w.barrier.get();
    a.info = info;
    a.maxit = o.maxit;
    a.eps = o.eps;
    a.ts = w.phase_ts;
    a.plan = plan_cg(A.wmax, 8);
    void *args[] = {&a};
    int G = cg_grid(A, a.plan, maxb);
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_cg_pipe, dim3(G), dim3(KBC), args, a.plan.smem, st)); ++::sysu::g_launches; }
}

void cg_solve_mixed(const SellDev &A, const double *val, const float *val32, const double *b, double *x,
                    bool x0_zero, const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = cg_max_blocks(k_cg_mixed_pipe);
    w.ensure(n, 1, maxb, st);
    w.ensure32(n, st);
    check_aligned16({x, val32, A.col.get(), w.r32.get(), w.z32.get(), w.p32.get(), w.q32.get(),
                     w.e32.get(), w.dinv32.get()});
    SellView V = view(A, val);
    { k_dinv32<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, w.dinv32.get()); ++::sysu::g_launches; }
    if (x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    CgPipeArgs a{};
    a.A = V;
    a.val32 = val32;
    a.b = b;
    a.x = x;
    a.r32 = w.r32.get();
    a.z32 = w.z32.get();
    a.p32 = w.p32.get();
    a.q32 = w.q32.get();
    a.e32 = w.e32.get();
    a.dinv32 = w.dinv32.get();
    a.partials = w.partials.get();
    a.gb = w.barrier.get();
    a.info = info;
    a.maxit = o.maxit;
    a.eps = o.eps;
    a.inner_tol = o.inner_tol;
    a.ts = w.phase_ts;
    a.plan = plan_cg(A.wmax, 4);
    void *args[] = {&a};
    int G = cg_grid(A, a.plan, maxb);
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_cg_mixed_pipe, dim3(G), dim3(KBC), args, a.plan.smem, st)); ++::sysu::g_launches; }
}

}  // namespace sysu
