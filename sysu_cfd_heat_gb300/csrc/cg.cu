// Jacobi-preconditioned CG on SELL-32 matrices: FP64, and FP32 recurrences
// with reliable FP64 updates.  Replaces LASPack's CGIter as the reference calls
// it for the pressure correction and the solid conduction equation
// (navier_pressure.cpp:29, HeatConductionSolver.cpp:90 through SolveLinearEqu,
// tools.cpp:56-64): same stopping test ||b - A x||_2 / ||b||_2 < eps, same
// iteration cap, and the iterates of Jacobi-PCG (Barrett et al., "Templates",
// Fig. 2.5) in exact arithmetic.
//
// One solve = one cooperative launch of a persistent kernel, one CTA per SM.
// Each CTA owns a contiguous range of slices (32-row groups of the SELL
// matrix).  An iteration is two phases, each closed by an exact grid
// reduction (exact_sum.cuh):
//   S  w = A z, p = z + beta p, q = w + beta q, p.q      (gathers z)
//   X  x += alpha p, r -= alpha q, z = M^-1 r, r.r, r.z
// S carries the direction update of Templates' loop (p = z + beta p) and keeps
// q = A p by the recurrence A (z + beta p) = A z + beta A p, so no separate grid
// barrier is needed between the direction update and the product.
//
// S streams the matrix: tiles of one slice per consumer warp (one row per
// consumer thread) are moved into shared memory by bulk asynchronous copies
// (cp.async.bulk, the TMA engine's 1-D form) through a ring of D slots.  The
// last warp is the producer: it issues a tile as soon as its slot has been
// released by all consumer warps, and queues the next iteration's first tiles
// at the start of X, so S starts on landed data.  In the FP64 kernel the
// consumers work one tile ahead (the next tile's gathers in flight during the
// current tile's FMAs: GB300's FP64 pipe, 1/64 of the FP32 rate, would
// otherwise idle while every warp waits on its gathers at once) -- except for
// large systems with rows of more than 5 entries, which measured faster one
// tile at a time on 1024 threads (cg_solve picks the form).  The matrix is copied with an L2
// evict-first policy so that the Krylov vectors stay in L2.  X runs over the
// CTA's rows with plain coalesced loads (all 32 warps, no per-tile
// synchronisation).
//
// Ring protocol (per CTA): tile job j lives in slot j % D; a slot's "full"
// mbarrier completes when its bytes land, its "empty" mbarrier when all
// consumer warps are done with it.  The producer warp runs converged (lane 0
// issues and takes the barrier decisions, broadcast by shuffle).  It blocks
// (bounded) only for tiles of the running S phase and otherwise issues only
// into free slots, so it always reaches the block barriers.  Only the matrix,
// which no kernel thread writes, goes through the async proxy.  Every wait is
// bounded; a CTA drains its copies before it leaves.
#include <climits>

#include "bulk.cuh"
#include "krylov_dev.cuh"

namespace sysu {
namespace {

// Threads per CTA (measured on the 2M-cell tet p' system: the FP64 kernel is
// fastest with 20 warps, 96 registers a thread and 608-row tiles -- 512 and 768
// threads measured 3-8 % slower -- the FP32 one with 24 warps and 736-row tiles).  The last warp produces, the others
// consume; a tile has one slice (32 rows) per consumer warp.
constexpr int CGT64 = 640;
// the look-ahead form for rows wider than 5 entries (hex) if it were used: on a 2.1M-cell
// hex cavity 640 threads measured 84.6 us per CG iteration, 512 threads 88.4 us, 7
// gathers held ahead the same as 6; the form without look-ahead on 1024 threads
// measured 82.3 us and is the one wide rows get (cg_solve)
constexpr int CGT64_WIDE = 640;
// threads of the FP64 CG instantiation that holds WR gathers a row ahead
template <int WR, bool AHEAD = true>
__host__ __device__ constexpr int cg64_threads() { return !AHEAD ? 1024 : (WR <= 5 ? CGT64 : CGT64_WIDE); }
constexpr int CGT32 = 768;
constexpr unsigned CG_SMEM_BUDGET = 200 * 1024;     // dynamic shared memory for the ring
constexpr int CG_WR = 6;                            // gathers per row held in registers one tile ahead (FP64)

// Launch plan: slices per tile, ring depth, slot size.
struct CgPlan {
    int ts = 1;
    int depth = 2;
    unsigned slot = 0;     // bytes per slot (multiple of 128)
    int direct = 0;        // 1: tiles read val/col from global memory (rows too long for a slot)
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
    // FP64 kernel behind a mixed solve: run only if gate->status[0] is
    // DEV_STALLED (the iterations of both are reported); null: always run
    const SolveInfo *gate;
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

// Consumer side of the ring (registers, uniform across the consumer warps).
struct Ring {
    int depth;
    unsigned slot;
    int cslot;          // slot of the next tile to consume
    unsigned cpar;      // its full-barrier phase parity
};
// Producer side (shared memory, read and written by the producer warp).
struct Producer {
    long long issued;   // tiles issued
    int nt;
    int islot;          // slot of the next tile to issue
    unsigned ipar;      // its round parity
    int itile;          // its tile
    int primed;         // tiles issued so far, saturating at depth
};
__shared__ Producer g_prod;

// First matrix entry of every tile of the CTA, so that issuing or reading a
// tile needs no global load of the slice pointers.
constexpr int CG_TILE_TABLE = 1024;
__shared__ int g_tile_e[CG_TILE_TABLE + 1];

__device__ __forceinline__ int tile_entry(const Part &P, const int *sl_ptr, int t) {
    return t <= CG_TILE_TABLE ? g_tile_e[t] : __ldg(sl_ptr + min(P.sb + t * P.ts, P.se));
}

__device__ __forceinline__ int cg_consumers() { return (int)(blockDim.x >> 5) - 1; }
__device__ __forceinline__ bool is_producer() { return (int)(threadIdx.x >> 5) == cg_consumers(); }

__device__ __forceinline__ unsigned char *cslot_ptr(const Ring &R) { return g_slots + (size_t)R.cslot * R.slot; }

// Producer warp (all 32 lanes, converged): issue tiles in order while slots
// are free; wait (bounded) for a slot only for tiles before `must_end`.  Lane 0
// issues the copies and takes the barrier decisions, broadcast to the warp.
// The state is worked on in registers (the copy instructions clobber memory).
template <class Issue>
__device__ __forceinline__ bool produce(const Ring &R, long long must_end, long long stop, Issue &&issue) {
    Producer &Q = g_prod;
    const bool lead = (threadIdx.x & 31) == 0;
    const int nt = Q.nt, depth = R.depth;
    long long issued = Q.issued;
    int islot = Q.islot, itile = Q.itile, primed = Q.primed;
    unsigned ipar = Q.ipar;
    const uint64_t pol = l2_policy_evict_first();
    bool ok = true;
    for (;;) {
        if (issued >= stop) break;
        if (primed == depth) {  // the slot's previous tile must be released by all consumers
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
        if (lead) issue(itile, g_slots + (size_t)islot * R.slot, &g_full[islot], pol);
        __syncwarp();
        if (++islot == depth) { islot = 0; ipar ^= 1u; }
        if (++itile == nt) itile = 0;
        ++issued;
    }
    __syncwarp();
    if (lead) {
        Q.issued = issued;
        Q.islot = islot;
        Q.ipar = ipar;
        Q.itile = itile;
        Q.primed = primed;
    }
    __syncwarp();
    return ok;
}

// Producer warp: the running S phase's tiles up to must_end (blocking) and
// whatever fits in free slots after them, never past tile job `stop`.
template <class Issue>
__device__ __forceinline__ void producer_tiles(const Ring &R, long long must_end, Issue &&issue, int *err,
                                               long long stop = LLONG_MAX) {
    if (!__all_sync(FULL_MASK, !fail_flag())) return;
    bool ok = produce(R, must_end, stop, issue);
    if (!ok && (threadIdx.x & 31) == 0) set_fail(err);
}

// Consumer warps: wait until the next tile has landed.  The outcome is uniform
// per warp; false after a timed-out wait (recorded in g_fail and *err).
__device__ __forceinline__ bool acquire(const Ring &R, int *err) {
    bool ok = !__any_sync(FULL_MASK, fail_flag() != 0);
    if (ok) ok = mbar_wait(&g_full[R.cslot], R.cpar);
    ok = __all_sync(FULL_MASK, ok);
    if (!ok && (threadIdx.x & 31) == 0) set_fail(err);
    return ok;
}

// As acquire/release, at an explicit slot (consumers that hold two tiles).
__device__ __forceinline__ bool acquire_at(int slot, unsigned par, int *err) {
    bool ok = !__any_sync(FULL_MASK, fail_flag() != 0);
    if (ok) ok = mbar_wait(&g_full[slot], par);
    ok = __all_sync(FULL_MASK, ok);
    if (!ok && (threadIdx.x & 31) == 0) set_fail(err);
    return ok;
}
__device__ __forceinline__ void release_at(int slot) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&g_empty[slot])) : "memory");
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
    if ((int)threadIdx.x != cg_consumers() * 32) return;
    long long issued = g_prod.issued;
    for (int s = 0; s < R.depth; ++s) {
        long long last = issued - 1 - ((issued - 1 - s) % R.depth + R.depth) % R.depth;
        if (last < 0) continue;
        if (!mbar_wait(&g_full[s], (unsigned)((last / R.depth) & 1))) break;
    }
}

__device__ __forceinline__ void ring_init(Ring &R, const CgPlan &pl, const Part &P, const int *sl_ptr) {
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
        Q.nt = nt;
        Q.islot = 0;
        Q.ipar = 0u;
        Q.itile = 0;
        Q.primed = 0;
        for (int k = 0; k < R.depth; ++k) {
            mbar_init(&g_full[k], 1);
            mbar_init(&g_empty[k], (unsigned)cg_consumers());
        }
        g_fail = 0;
        mbar_init_fence();
    }
    __syncthreads();
}

// Loop state code from the squared residual: 1 converged (||r||^2 < thr,
// thr = eps^2 ||b||^2, the stopping test ||r|| / ||b|| < eps without a square
// root or division per iteration), 2 not finite, 0 go on.
__device__ __forceinline__ double stop_code(double rr, double thr) {
    return rr < thr ? 1.0 : (isfinite(rr) ? 0.0 : 2.0);
}

// One SELL row of a tile: the column indices of up to 8 entries, then their
// gathers, then the FMAs.  diag = x of the row itself (entry 0 is the diagonal).
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

// The tile copy of the matrix (values, then the column indices) for tile t.
template <class V>
__device__ __forceinline__ void issue_matrix_tile(const Part &P, const SellView &A, const V *val, int direct, int t,
                                                  unsigned char *dst, uint64_t *bar, uint64_t pol) {
    if (direct) {
        mbar_arrive_expect_tx(bar, 0);
        return;
    }
    long e0 = tile_entry(P, A.sl_ptr, t), e1 = tile_entry(P, A.sl_ptr, t + 1);
    unsigned bv = (unsigned)((e1 - e0) * sizeof(V)), bc = (unsigned)((e1 - e0) * 4);
    mbar_arrive_expect_tx(bar, bv + bc);
    if (bv) {
        bulk_g2s(dst, val + e0, bv, bar, pol);
        bulk_g2s(dst + bv, A.col + e0, bc, bar, pol);
    }
}

// X phase over the CTA's rows: x += alpha p, r -= alpha q, z = M^-1 r and the
// thread's partial r.r and r.z.  RB rows per thread per step with all their
// loads issued before the arithmetic (the buffers are distinct, so the loads of
// a step need not wait for the stores of the previous one); the partial sums
// take the rows in the same order as a one-row loop.  (Holding the next step's
// loads in flight during the current step's arithmetic measured no faster.)
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// |r| 2^-k as an FP32 number made from r's high word with integer operations only
// (20 of the 52 mantissa bits, relative error below 2^-20): GB300's FP64 pipe runs
// at 1/64 of the FP32 rate, and r.r serves only the stopping test.  bias = 1023 +
// k - 127.  Exponent 0x7FF (inf, NaN) gives NaN; values below FP32's normal range
// give 0; huge ones are held at 2^50 so that a thread's sum of squares stays finite.
__device__ __forceinline__ float scaled_abs_f32(double r, int bias) {
    const int hi = __double2hiint(r);
    const int e = (hi >> 20) & 0x7FF;
    if (e == 0x7FF) return __int_as_float(0x7FC00000);
    const int fe = e - bias;
    if (fe <= 0) return 0.f;
    return __int_as_float((min(fe, 127 + 50) << 23) | ((hi & 0xFFFFF) << 3));
}

// X phase of the FP64 kernel with r.r estimated in FP32 (rr32, in units of 2^-2k);
// x, r, z and r.z exactly as x_phase computes them.
template <int NT, int RB>
__device__ __forceinline__ void x_phase_est(int R0, int R1, double alpha, const double *__restrict__ pv,
                                            const double *__restrict__ qv, const double *__restrict__ dv,
                                            double *__restrict__ xv, double *__restrict__ rv,
                                            double *__restrict__ zv, float &rr32, double &rz, int bias) {
    int i = R0 + (int)threadIdx.x;
    for (; i + (RB - 1) * NT < R1; i += RB * NT) {
        double p[RB], q[RB], x[RB], r[RB], d[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int j = i + u * NT;
            p[u] = pv[j];
            q[u] = qv[j];
            x[u] = xv[j];
            r[u] = rv[j];
            d[u] = dv[j];
        }
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int j = i + u * NT;
            x[u] = fma_t(alpha, p[u], x[u]);
            r[u] = fma_t(-alpha, q[u], r[u]);
            const double z = d[u] * r[u];
            xv[j] = x[u];
            rv[j] = r[u];
            zv[j] = z;
            const float f = scaled_abs_f32(r[u], bias);
            rr32 = fmaf(f, f, rr32);
            rz = fma_t(r[u], z, rz);
        }
    }
    for (; i < R1; i += NT) {
        double pi = pv[i], qi = qv[i], xi = xv[i], ri = rv[i], di = dv[i];
        xi = fma_t(alpha, pi, xi);
        ri = fma_t(-alpha, qi, ri);
        const double zi = di * ri;
        xv[i] = xi;
        rv[i] = ri;
        zv[i] = zi;
        const float f = scaled_abs_f32(ri, bias);
        rr32 = fmaf(f, f, rr32);
        rz = fma_t(ri, zi, rz);
    }
}

template <class T, int NT, int RB>
__device__ __forceinline__ void x_phase(int R0, int R1, T alpha, const T *__restrict__ pv, const T *__restrict__ qv,
                                        const T *__restrict__ dv, T *__restrict__ xv, T *__restrict__ rv,
                                        T *__restrict__ zv, T &rr, T &rz) {
    int i = R0 + (int)threadIdx.x;
    for (; i + (RB - 1) * NT < R1; i += RB * NT) {
        T p[RB], q[RB], x[RB], r[RB], d[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int j = i + u * NT;
            p[u] = pv[j];
            q[u] = qv[j];
            x[u] = xv[j];
            r[u] = rv[j];
            d[u] = dv[j];
        }
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int j = i + u * NT;
            x[u] = fma_t(alpha, p[u], x[u]);
            r[u] = fma_t(-alpha, q[u], r[u]);
            const T z = d[u] * r[u];
            xv[j] = x[u];
            rv[j] = r[u];
            zv[j] = z;
            rr = fma_t(r[u], r[u], rr);
            rz = fma_t(r[u], z, rz);
        }
    }
    for (; i < R1; i += NT) {
        T pi = pv[i], qi = qv[i], xi = xv[i], ri = rv[i], di = dv[i];
        xi = fma_t(alpha, pi, xi);
        ri = fma_t(-alpha, qi, ri);
        const T zi = di * ri;
        xv[i] = xi;
        rv[i] = ri;
        zv[i] = zi;
        rr = fma_t(ri, ri, rr);
        rz = fma_t(ri, zi, rz);
    }
}

// Consumer warps over the CTA's tiles, one row per thread per tile: w = A z for
// the row, then epi(i, w, z_i, p_i, q_i) (p_i, q_i loaded when has_dir).  One
// tile ahead: tile t+1's row loads and its first WR gathers are in flight
// while tile t's FMAs run, so the arithmetic of one tile overlaps the memory
// latency of the next (the warp holds two slots).  val: the matrix values of
// this precision (read from global memory in direct mode).  The FMAs take a
// row's entries in order, the first as a product, as tile_row_dot does.
template <class V, int WR, class Epi, bool AHEAD = true>
__device__ __forceinline__ void tiles_ahead(const Part &P, Ring &R, const SellView &A, const V *val, int direct,
                                            const V *pv, const V *qv, const V *__restrict__ zv, bool has_dir,
                                            int *err, Epi &&epi) {
    const int tid = threadIdx.x;
    const int nt = P.nt;
    int aslot = R.cslot;  // acquire cursor
    unsigned apar = R.cpar;
    int rslot = R.cslot;  // release cursor
    V zc[WR], zn[WR];
    V pc = 0, qc = 0, pn = 0, qn = 0;
    int ec = 0, wc = 0, en = 0, wn = 0;
    // row loads, tile wait, column reads and gathers of tile t
    auto fetch = [&](int t, V(&zz)[WR], V &pp, V &qq, int &ee, int &ww) -> bool {
        int s0, s1, r0, nr;
        P.tile(t, s0, s1, r0, nr);
        const bool act = tid < nr;
        const int i = r0 + tid;
        const int s = s0 + (tid >> 5);
        pp = qq = 0;
        ee = ww = 0;
        if (act) {
            if (has_dir) { pp = pv[i]; qq = qv[i]; }
            ee = __ldg(A.sl_ptr + s);
            ww = __ldg(A.sl_w + s);
        }
        if (!acquire_at(aslot, apar, err)) return false;
        const unsigned char *slot = g_slots + (size_t)aslot * R.slot;
        if (++aslot == R.depth) { aslot = 0; apar ^= 1u; }
        if (act) {
            const int e0 = tile_entry(P, A.sl_ptr, t), e1 = tile_entry(P, A.sl_ptr, t + 1);
            ee = ee - e0 + (tid & 31);
            const int *cs = direct ? A.col + e0 : reinterpret_cast<const int *>(slot + (size_t)(e1 - e0) * sizeof(V));
            int c[WR];
#pragma unroll
            for (int k = 0; k < WR; ++k)
                if (k < ww) c[k] = cs[ee + 32 * k];
#pragma unroll
            for (int k = 0; k < WR; ++k)
                if (k < ww) zz[k] = zv[c[k]];
        }
        return true;
    };
    // the FMAs of tile t, then its slot is released
    auto finish = [&](int t, const V(&zz)[WR], V pp, V qq, int ee, int ww) {
        int s0, s1, r0, nr;
        P.tile(t, s0, s1, r0, nr);
        if (tid < nr) {
            const int i = r0 + tid;
            const int e0 = tile_entry(P, A.sl_ptr, t), e1 = tile_entry(P, A.sl_ptr, t + 1);
            const unsigned char *slot = g_slots + (size_t)rslot * R.slot;
            const V *vs = direct ? val + e0 : reinterpret_cast<const V *>(slot);
            const int *cs = direct ? A.col + e0 : reinterpret_cast<const int *>(slot + (size_t)(e1 - e0) * sizeof(V));
            V acc = 0, zi = 0;
            if (ww > 0) {
                acc = vs[ee] * zz[0];
                zi = zz[0];
            }
#pragma unroll
            for (int k = 1; k < WR; ++k)
                if (k < ww) acc = fma_t(vs[ee + 32 * k], zz[k], acc);
            for (int k = WR; k < ww; ++k) acc = fma_t(vs[ee + 32 * k], zv[cs[ee + 32 * k]], acc);
            epi(i, acc, zi, pp, qq);
        }
        release_at(rslot);
        if (++rslot == R.depth) rslot = 0;
    };
    if (!AHEAD) {  // one tile at a time: fetch, then the FMAs (fewer registers)
        for (int t = 0; t < nt; ++t) {
            if (!fetch(t, zc, pc, qc, ec, wc)) break;
            finish(t, zc, pc, qc, ec, wc);
        }
        R.cslot = aslot;
        R.cpar = apar;
        return;
    }
    bool ok = nt > 0 && fetch(0, zc, pc, qc, ec, wc);
    for (int t = 0; ok && t < nt; ++t) {
        if (t + 1 < nt && !fetch(t + 1, zn, pn, qn, en, wn)) break;
        finish(t, zc, pc, qc, ec, wc);
#pragma unroll
        for (int k = 0; k < WR; ++k) zc[k] = zn[k];
        pc = pn;
        qc = qn;
        ec = en;
        wc = wn;
    }
    R.cslot = aslot;
    R.cpar = apar;
}

// S phase of one CG iteration for a consumer warp: w = A z, p = z + beta p,
// q = w + beta q; returns the thread's partial p.q.
template <class V, int WR, bool AHEAD = true>
__device__ __forceinline__ V s_phase(const Part &P, Ring &R, const SellView &A, const V *val, int direct,
                                     V *__restrict__ pv, V *__restrict__ qv, const V *__restrict__ zv, V beta,
                                     bool has_dir, int *err) {
    V pq = 0;
    auto epi = [&](int i, V w, V zi, V pp, V qq) {
        pp = fma_t(beta, pp, zi);
        qq = fma_t(beta, qq, w);
        pv[i] = pp;
        qv[i] = qq;
        pq = fma_t(pp, qq, pq);
    };
    tiles_ahead<V, WR, decltype(epi) &, AHEAD>(P, R, A, val, direct, pv, qv, zv, has_dir, err, epi);
    return pq;
}

// ---------------------------------------------------------------------------
// FP64
// WR: gathers per row held in registers (one tile ahead when AHEAD): 5 for rows of at
// most 5 entries (tets), else CG_WR
template <int WR, bool AHEAD = true>
__global__ void __launch_bounds__(cg64_threads<WR, AHEAD>(), 1) k_cg_pipe(CgPipeArgs a) {
    constexpr int NT = cg64_threads<WR, AHEAD>();
    if (a.gate && a.gate->status[0] != DEV_STALLED) return;  // the same word for every block
    const int it_before = a.gate ? a.gate->iters[0] : 0;
    const int n = a.A.n;
    const int tid = threadIdx.x;
    const bool prod = is_producer();
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const Part P = make_part(n, a.A.nslices, a.plan.ts);
    const int nt = P.nt;
    const int R0 = P.sb * 32, R1 = min(P.se * 32, n);
    Ring R;
    ring_init(R, a.plan, P, a.A.sl_ptr);
    auto issue = [&](int t, unsigned char *dst, uint64_t *bar, uint64_t pol) {
        issue_matrix_tile<double>(P, a.A, a.A.val, a.plan.direct, t, dst, bar, pol);
    };
    if (prod) producer_tiles(R, 0, issue, err);  // the first tiles land during the initial residual

    // r = b - A x, z = M^-1 r; ||b||^2, ||r||^2, r.z
    double v3[3] = {0.0, 0.0, 0.0};
    for (int i = R0 + tid; i < R1; i += NT) {
        double bi = a.b[i];
        double ri = bi - row_dot(a.A, i, a.x);
        double zi = a.dinv[i] * ri;
        a.r[i] = ri;
        a.z[i] = zi;
        v3[0] = fma(bi, bi, v3[0]);
        v3[1] = fma(ri, ri, v3[1]);
        v3[2] = fma(ri, zi, v3[2]);
    }
    if (!grid_sum_t0<3>(v3, rc, a.gb, err)) { drain(R); return; }
    // thread-0 scalar state, kept in shared memory (no registers in the other threads)
    __shared__ double s_state[5];
    double &bb = s_state[0], &rr = s_state[1], &rho = s_state[2], &thr = s_state[3], &est_unit = s_state[4];
    __shared__ int s_bias, s_rr_est;  // scaling of the r.r estimate (0: exact r.r); rr holds an estimate
    if (tid == 0) {
        bb = v3[0] == 0.0 ? 1.0 : v3[0];
        thr = a.eps * a.eps * bb;
        rr = v3[1];
        rho = v3[2];
        g_bc[0] = stop_code(rr, thr);
        g_bc[1] = 0.0;
        // estimate r.r in FP32 in units of 2^2k, 2^2k ~ thr (0: thr unusable, exact r.r)
        s_bias = 0;
        s_rr_est = 0;
        if (thr > 0.0 && isfinite(thr)) {
            const int e = ilogb(thr);
            const int k = e >= 0 ? e / 2 : -((1 - e) / 2);  // floor(e / 2)
            if (k > -900 && k < 900) {
                s_bias = 1023 + k - 127;
                est_unit = ldexp(1.0, 2 * k);
            }
        }
    }
    __syncthreads();
    const int rr_bias = s_bias;

    long long base = 0;  // job index of the running S phase's first tile
    int it = 0, status = DEV_OK;
    for (;;) {
        double code = g_bc[0], beta = g_bc[1];
        __syncthreads();
        if (code == 1.0 || it >= a.maxit) break;
        if (code == 2.0) { status = DEV_NONFINITE; break; }
        ++it;
        stamp(a.ts, it, 0);
        // S: w = A z, p = z + beta p, q = w + beta q, p.q
        double v1[1] = {0.0};
        if (prod) {
            producer_tiles(R, base + nt, issue, err);
        } else {
            v1[0] = s_phase<double, WR, AHEAD>(P, R, a.A, a.A.val, a.plan.direct, a.p, a.q, a.z, beta, it > 1, err);
        }
        base += nt;
        if (!grid_sum_t0<1>(v1, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, it, 1);
        if (tid == 0) {
            g_bc[2] = v1[0] == 0.0 ? 0.0 : rho / v1[0];
            g_bc[3] = v1[0] == 0.0 ? 1.0 : 0.0;
        }
        __syncthreads();
        double alpha = g_bc[2];
        if (g_bc[3] != 0.0) { status = DEV_BREAKDOWN; break; }
        // X: the producer first queues the next S phase's tiles
        if (prod) producer_tiles(R, 0, issue, err);
        double v2[2] = {0.0, 0.0};
        if (rr_bias) {
            float rr32 = 0.f;
            x_phase_est<NT, 4>(R0, R1, alpha, a.p, a.q, a.dinv, a.x, a.r, a.z, rr32, v2[1], rr_bias);
            v2[0] = (double)rr32;
        } else {
            x_phase<double, NT, 4>(R0, R1, alpha, a.p, a.q, a.dinv, a.x, a.r, a.z, v2[0], v2[1]);
        }
        if (!grid_sum_t0<2>(v2, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, it, 2);
        if (tid == 0) {
            g_bc[1] = v2[1] / rho;
            rho = v2[1];
            if (rr_bias) {
                // the estimate decides only when it is clearly above the threshold
                rr = v2[0] * est_unit;
                s_rr_est = 1;
                g_bc[5] = rr >= thr * 1.001 ? 0.0 : 1.0;  // 1: take the exact r.r (NaN included)
                g_bc[0] = 0.0;
            } else {
                rr = v2[0];
                g_bc[0] = stop_code(rr, thr);
                g_bc[5] = 0.0;
            }
        }
        __syncthreads();
        if (g_bc[5] != 0.0) {  // near (or below) the threshold: the exact FP64 r.r
            double e1[1] = {0.0};
            for (int i = R0 + tid; i < R1; i += NT) e1[0] = fma(a.r[i], a.r[i], e1[0]);
            if (!grid_sum_t0<1>(e1, rc, a.gb, err)) break;
            if (tid == 0) {
                rr = e1[0];
                s_rr_est = 0;
                g_bc[0] = stop_code(rr, thr);
            }
            __syncthreads();
        }
    }
    drain(R);
    // the reported residual is the exact one: recompute r.r if rr holds an estimate
    // (not after a failed wait, when the blocks no longer meet)
    if (s_rr_est && !fail_flag() && !(a.info->err)) {
        double e1[1] = {0.0};
        for (int i = R0 + tid; i < R1; i += NT) e1[0] = fma(a.r[i], a.r[i], e1[0]);
        if (grid_sum_t0<1>(e1, rc, a.gb, err) && tid == 0) rr = e1[0];
        __syncthreads();
    }
    if (blockIdx.x == 0 && tid == 0) {
        double res = sqrt(rr) / sqrt(bb);
        if (status == DEV_OK && !(rr < thr)) status = isfinite(rr) ? DEV_MAXITER : DEV_NONFINITE;
        a.info->status[0] = status;
        a.info->iters[0] = it_before + it;
        a.info->res[0] = res;
    }
}

// ---------------------------------------------------------------------------
// Mixed precision: the recurrences (p, q, r, z and the correction e) run in
// FP32, with reliable updates (Sleijpen & van der Vorst, "Reliable updated
// residuals in hybrid Bi-CG methods", Computing 56, 1996): once the FP32
// residual has fallen by inner_tol since the last update, e is added to the
// FP64 solution, e is zeroed, the FP64 residual b - A x replaces the FP32 one
// and the search direction is kept, so the Krylov process is not restarted --
// unless that FP64 residual norm has not halved since the previous update
// (near FP32's rounding floor at tight tolerances), when it restarts from z.
// Convergence is decided on that FP64 residual only.  Per-thread partial dot
// products run in FP32 over the thread's rows; exact sums across threads.
__global__ void __launch_bounds__(CGT32, 1) k_cg_mixed_pipe(CgPipeArgs a) {
    const int n = a.A.n;
    const int tid = threadIdx.x;
    const bool prod = is_producer();
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const Part P = make_part(n, a.A.nslices, a.plan.ts);
    const int nt = P.nt;
    const int R0 = P.sb * 32, R1 = min(P.se * 32, n);
    const float *__restrict__ dinv = a.dinv32;
    Ring R;
    ring_init(R, a.plan, P, a.A.sl_ptr);
    auto issue = [&](int t, unsigned char *dst, uint64_t *bar, uint64_t pol) {
        issue_matrix_tile<float>(P, a.A, a.val32, a.plan.direct, t, dst, bar, pol);
    };
    if (prod) producer_tiles(R, 0, issue, err);

    // FP64 residual of the initial guess (kept in a.r), then its FP32 copy scaled
    // by a power of two sig to norm ~1: the FP32 process runs in sig units
    double v2i[2] = {0.0, 0.0};
    for (int i = R0 + tid; i < R1; i += CGT32) {
        double bi = a.b[i];
        double ri = bi - row_dot(a.A, i, a.x);
        a.r[i] = ri;
        v2i[0] = fma(bi, bi, v2i[0]);
        v2i[1] = fma(ri, ri, v2i[1]);
    }
    if (!grid_sum_t0<2>(v2i, rc, a.gb, err)) { drain(R); return; }
    // thread-0 scalar state, kept in shared memory (no registers in the other threads);
    // rr_ref: FP64 ||b - A x||^2 at the last reliable update; sig: the scale of the
    // FP32 vectors (r32 = sig r), sig_next: the scale after the next update
    __shared__ double s_state[6];
    __shared__ int s_stalls;  // consecutive updates that did not halve the FP64 residual norm
    double &bb = s_state[0], &thr = s_state[1], &rho = s_state[2], &rr_ref = s_state[3], &sig = s_state[4],
           &sig_next = s_state[5];
    if (tid == 0) {
        bb = v2i[0] == 0.0 ? 1.0 : v2i[0];
        thr = a.eps * a.eps * bb;
        rr_ref = v2i[1];
        sig = pow2_scale(rr_ref);
        s_stalls = 0;
        g_bc[5] = sig;
    }
    __syncthreads();
    {
        const double sg = g_bc[5];
        float f2 = 0.f;
        for (int i = R0 + tid; i < R1; i += CGT32) {
            float rf = (float)(sg * a.r[i]), zf = dinv[i] * rf;
            a.r32[i] = rf;
            a.z32[i] = zf;
            a.e32[i] = 0.f;
            f2 = fmaf(rf, zf, f2);
        }
        double v1[1] = {(double)f2};
        if (!grid_sum_t0<1>(v1, rc, a.gb, err)) { drain(R); return; }
        if (tid == 0) {
            rho = v1[0];
            g_bc[0] = stop_code(rr_ref, thr);
            g_bc[1] = 0.0;
        }
        __syncthreads();
    }

    long long base = 0;
    int total = 0, nupd = 0, status = DEV_OK;
    for (;;) {
        double code = g_bc[0];  // from the FP64 residual of the last update
        float beta = (float)g_bc[1];
        __syncthreads();
        if (code == 1.0 || total >= a.maxit) break;
        if (code == 2.0) { status = DEV_NONFINITE; break; }
        if (code == 3.0) { status = DEV_STALLED; break; }
        ++total;
        stamp(a.ts, total, 0);
        float g0 = 0.f;
        if (prod) {
            producer_tiles(R, base + nt, issue, err);
        } else {
            // one tile at a time: the look-ahead of s_phase measured slower here (FP32
            // arithmetic is cheap, and its registers spill at 768 threads)
            for (int t = 0; t < nt; ++t) {
                int s0, s1, r0, nr;
                P.tile(t, s0, s1, r0, nr);
                const bool act = tid < nr;
                const int i = r0 + tid;
                const int s = s0 + (tid >> 5);
                float pi = 0.f, qi = 0.f;
                int es = 0, w = 0;
                if (act) {
                    if (total > 1) { pi = a.p32[i]; qi = a.q32[i]; }
                    es = __ldg(a.A.sl_ptr + s);
                    w = __ldg(a.A.sl_w + s);
                }
                if (!acquire(R, err)) break;
                if (act) {
                    int e0 = tile_entry(P, a.A.sl_ptr, t), e1 = tile_entry(P, a.A.sl_ptr, t + 1);
                    es = es - e0 + (tid & 31);
                    const float *vs;
                    const int *cs;
                    if (a.plan.direct) {
                        vs = a.val32 + e0;
                        cs = a.A.col + e0;
                    } else {
                        vs = reinterpret_cast<const float *>(cslot_ptr(R));
                        cs = reinterpret_cast<const int *>(cslot_ptr(R) + (size_t)(e1 - e0) * 4);
                    }
                    float zi;
                    float wi = tile_row_dot<float, float, float>(vs, cs, es, w, a.z32, zi);
                    pi = fmaf(beta, pi, zi);
                    qi = fmaf(beta, qi, wi);
                    a.p32[i] = pi;
                    a.q32[i] = qi;
                    g0 = fmaf(pi, qi, g0);
                }
                release(R);
            }
        }
        base += nt;
        double v1[1] = {(double)g0};
        if (!grid_sum_t0<1>(v1, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, total, 1);
        if (tid == 0) {
            g_bc[2] = v1[0] == 0.0 ? 0.0 : rho / v1[0];
            g_bc[3] = v1[0] == 0.0 ? 1.0 : 0.0;
        }
        __syncthreads();
        float alpha = (float)g_bc[2];
        if (g_bc[3] != 0.0) { status = DEV_BREAKDOWN; break; }
        if (prod) producer_tiles(R, 0, issue, err);
        float h0 = 0.f, h1 = 0.f;
        x_phase<float, CGT32, 4>(R0, R1, alpha, a.p32, a.q32, dinv, a.e32, a.r32, a.z32, h0, h1);
        double w2[2] = {(double)h0, (double)h1};
        if (!grid_sum_t0<2>(w2, rc, a.gb, err) || fail_flag()) break;
        stamp(a.ts, total, 2);
        if (tid == 0) {
            // reliable update once the FP32 residual fell by inner_tol since the
            // last one, when it looks converged, or at the iteration cap
            // (the FP32 sums are in sig^2 units)
            const double d2 = a.inner_tol * a.inner_tol, s2 = sig * sig;
            bool upd = w2[0] <= d2 * rr_ref * s2 || w2[0] <= thr * s2 || total >= a.maxit || !(w2[0] == w2[0]);
            if (!upd) {
                g_bc[1] = w2[1] / rho;
                rho = w2[1];
            } else {
                // the next scale from the FP32 estimate of the new residual
                sig_next = sig * pow2_scale(w2[0]);
                g_bc[5] = 1.0 / sig;  // x += e / sig (a power of two: exact)
                g_bc[6] = sig_next;
            }
            g_bc[4] = upd ? 1.0 : 0.0;
        }
        __syncthreads();
        if (g_bc[4] != 0.0) {
            const double isg = g_bc[5], sn = g_bc[6];
            for (int i = R0 + tid; i < R1; i += CGT32) {
                a.x[i] += (double)a.e32[i] * isg;
                a.e32[i] = 0.f;
            }
            if (!grid_sync(a.gb, err)) break;
            double u[2] = {0.0, 0.0};
            float fz = 0.f;
            for (int i = R0 + tid; i < R1; i += CGT32) {
                double ri = a.b[i] - row_dot(a.A, i, a.x);
                float rf = (float)(sn * ri), zf = dinv[i] * rf;
                a.r32[i] = rf;
                a.z32[i] = zf;
                u[0] = fma(ri, ri, u[0]);
                fz = fmaf(rf, zf, fz);
            }
            u[1] = (double)fz;
            if (!grid_sum_t0<2>(u, rc, a.gb, err)) break;
            if (tid == 0) {
                // keep the direction (beta from the replaced residual) while the
                // updates make progress; once the FP64 residual norm has not at
                // least halved since the last update (the FP32 recurrence has met
                // its rounding floor), restart it from z: beta = 0
                // beta in the new units: (rho_new / rho_old) (sig / sig_next), so
                // that the kept p and q (in sig units) scale with the new r
                const bool stalled = !(u[0] < 0.25 * rr_ref);
                s_stalls = stalled ? s_stalls + 1 : 0;
                rr_ref = u[0];
                g_bc[0] = stop_code(rr_ref, thr);
                if (g_bc[0] == 0.0 && s_stalls >= 3) g_bc[0] = 3.0;  // hand over to FP64
                g_bc[1] = stalled ? 0.0 : (u[1] / rho) * (sig / sig_next);
                rho = u[1];
                sig = sig_next;
                ++nupd;
            }
            __syncthreads();
        }
    }
    drain(R);
    if (status == DEV_BREAKDOWN) {  // keep the correction gathered so far
        const double isg = 1.0 / s_state[4];
        for (int i = R0 + tid; i < R1; i += CGT32) a.x[i] += (double)a.e32[i] * isg;
    }
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

// ---------------------------------------------------------------------------
// Standalone y = A x with the matrix streamed through the same ring (the SpMV
// of the sweep): one CTA per SM, the producer issues each of the CTA's tiles
// once, the consumers gather x one tile ahead.
template <class V>
__global__ void __launch_bounds__(CGT64, 1) k_spmv_ring(SellView A, const V *val, const V *x, V *y, CgPlan plan,
                                                       int *err) {
    const Part P = make_part(A.n, A.nslices, plan.ts);
    Ring R;
    ring_init(R, plan, P, A.sl_ptr);
    auto issue = [&](int t, unsigned char *dst, uint64_t *bar, uint64_t pol) {
        issue_matrix_tile<V>(P, A, val, plan.direct, t, dst, bar, pol);
    };
    if (is_producer()) {
        producer_tiles(R, P.nt, issue, err, P.nt);
    } else {
        tiles_ahead<V, CG_WR>(P, R, A, val, plan.direct, nullptr, nullptr, x, false, err,
                       [&](int i, V w, V, V, V) { y[i] = w; });
    }
    drain(R);
}

// Tile size and ring depth for a matrix whose widest slice has wmax entries
// per row; ebytes = bytes per matrix value.
CgPlan plan_cg(int wmax, int ebytes, int consumers) {
    CgPlan pl;
    auto round128 = [](unsigned b) { return (b + 127u) & ~127u; };
    for (int ts = consumers; ts >= 1; ts /= 2) {
        unsigned slot = round128((unsigned)ts * 32 * (unsigned)std::max(wmax, 1) * (unsigned)(ebytes + 4));
        int depth = (int)std::min<unsigned>(CopyRing::DMAX, CG_SMEM_BUDGET / slot);
        if (depth >= 2) {
            pl.ts = ts;
            pl.depth = depth;
            pl.slot = slot;
            pl.smem = slot * depth;
            return pl;
        }
    }
    // rows too long for a slot: tiles read the matrix from global memory
    pl.ts = consumers;
    pl.direct = 1;
    pl.slot = 128;
    pl.depth = 2;
    pl.smem = pl.slot * pl.depth;
    return pl;
}

template <class K>
int cg_max_blocks(K kernel, int threads) {
    SYSU_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CG_SMEM_BUDGET));
    int per_sm = 0;
    SYSU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, CG_SMEM_BUDGET));
    if (per_sm < 1) throw CaseError{"persistent CG kernel cannot be resident"};
    return per_sm * num_sms();
}

int cg_grid(const SellDev &A, const CgPlan &pl, int maxb, int sm_cap) {
    if (sm_cap > 0) maxb = std::min(maxb, sm_cap * std::max(1, maxb / num_sms()));
    int tiles = (A.nslices + pl.ts - 1) / pl.ts;
    return std::max(1, std::min(tiles, maxb));
}

}  // namespace

// The FP64 persistent CG.  gate: see CgPipeArgs (then x is not zeroed and
// info is not cleared: the solve continues the mixed one's).
static void cg_launch64(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
                        const KrylovOpts &o, KrylovWork &w, SolveInfo *info, const SolveInfo *gate,
                        cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    // rows of at most 5 entries (tets): 5 gathers held one tile ahead on 640 threads
    // (2.5 % faster than 6 on the 2M-cell tet p' system); wider rows (hex: 7): one tile
    // at a time on 1024 threads (3 % faster there than the look-ahead form)
    // (below 1M rows the wide form also looks ahead: the 256k-row hex p' system of the
    // CHT channel is latency-bound and measured 7.99 ms per solve that way, 8.37 ms
    // one tile at a time)
    const bool narrow = A.wmax <= 5, wide_big = !narrow && n >= (1 << 20);
    auto kern = narrow ? k_cg_pipe<5, true> : (wide_big ? k_cg_pipe<CG_WR, false> : k_cg_pipe<CG_WR, true>);
    static int maxb5 = 0, maxb6 = 0, maxb6a = 0;
    int &maxb = narrow ? maxb5 : (wide_big ? maxb6 : maxb6a);
    const int nthreads = narrow ? cg64_threads<5, true>()
                                : (wide_big ? cg64_threads<CG_WR, false>() : cg64_threads<CG_WR, true>());
    if (!maxb) maxb = cg_max_blocks(kern, nthreads);
    w.ensure(n, 1, maxb, st);
    check_aligned16({val, A.col.get()});
    SellView V = view(A, val);
    { k_jacobi_dinv<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, o.jacobi ? 1 : 0, w.dinv.get()); ++::sysu::g_launches; }
    if (!gate && x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    if (!gate) SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    CgPipeArgs a{};
    a.gate = gate;
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
    a.plan = plan_cg(A.wmax, 8, nthreads / 32 - 1);
    void *args[] = {&a};
    int G = cg_grid(A, a.plan, maxb, w.sm_cap);
    SYSU_CUDA(cudaMemsetAsync(w.barrier.get(), 0, sizeof(GridBarrier), st));  // grid_sync starts from 0
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)kern, dim3(G), dim3(nthreads), args, a.plan.smem, st)); ++::sysu::g_launches; }
}

void cg_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
              const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    cg_launch64(A, val, b, x, x0_zero, o, w, info, nullptr, st);
}

template <class V>
static void spmv_ring_t(const SellDev &A, const V *val, const V *x, V *y, int *err, cudaStream_t st) {
    if (A.n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = cg_max_blocks(k_spmv_ring<V>, CGT64);
    check_aligned16({val, A.col.get()});
    const CgPlan pl = plan_cg(A.wmax, (int)sizeof(V), CGT64 / 32 - 1);
    const int G = cg_grid(A, pl, maxb, 0);
    SellView Av = view(A, nullptr);
    k_spmv_ring<V><<<G, CGT64, pl.smem, st>>>(Av, val, x, y, pl, err);
    ++::sysu::g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void spmv_ring(const SellDev &A, const double *val, const double *x, double *y, int *err, cudaStream_t st) {
    spmv_ring_t<double>(A, val, x, y, err, st);
}

void spmv_ring32(const SellDev &A, const float *val, const float *x, float *y, int *err, cudaStream_t st) {
    spmv_ring_t<float>(A, val, x, y, err, st);
}

void cg_solve_mixed(const SellDev &A, const double *val, const float *val32, const double *b, double *x,
                    bool x0_zero, const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = cg_max_blocks(k_cg_mixed_pipe, CGT32);
    w.ensure(n, 1, maxb, st);
    w.ensure32(n, st);
    check_aligned16({val32, A.col.get()});
    SellView V = view(A, val);
    { k_dinv32<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, w.dinv32.get()); ++::sysu::g_launches; }
    if (x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    CgPipeArgs a{};
    a.A = V;
    a.val32 = val32;
    a.b = b;
    a.x = x;
    a.r = w.r.get();  // FP64 initial residual
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
    a.plan = plan_cg(A.wmax, 4, CGT32 / 32 - 1);
    void *args[] = {&a};
    int G = cg_grid(A, a.plan, maxb, w.sm_cap);
    SYSU_CUDA(cudaMemsetAsync(w.barrier.get(), 0, sizeof(GridBarrier), st));  // grid_sync starts from 0
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_cg_mixed_pipe, dim3(G), dim3(CGT32), args, a.plan.smem, st)); ++::sysu::g_launches; }
    // FP64 takes over from the current x if the FP32 refinement stalled (the
    // launch returns at once otherwise).  Not for solves capped to a share of
    // the SMs (cases of one CUDA graph): there a cooperative launch that needs
    // whole SMs waits for room and holds up the graph's other branches, and a
    // stalled solve reports DEV_STALLED instead.
    if (w.sm_cap <= 0) cg_launch64(A, val, b, x, false, o, w, info, info, st);
}

}  // namespace sysu
