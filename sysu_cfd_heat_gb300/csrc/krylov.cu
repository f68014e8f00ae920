// Persistent cooperative Krylov solvers on SELL-32 matrices (FP64): BiCGSTAB
// for one or three right-hand sides, and the standalone SpMV / Jacobi kernels.
// The CG family lives in cg.cu.
//
// One solve = one cooperative launch.  Rows are distributed thread-per-row with
// a grid stride that is a multiple of 32, so each warp owns whole slices.
// Global dot products are reduced deterministically: warp shuffles, then the
// block, then every block sums the per-block partials in the same fixed order,
// so all blocks take identical convergence decisions and repeated runs are
// bit-identical.  Every barrier wait is bounded (device.hpp).
//
// Algorithm (restated from Barrett et al., "Templates", Fig. 2.10; the same
// recurrences as the CPU oracle's LASPack restatement): BiCGSTAB, right
// preconditioned, early exit on ||s||, breakdown on rho = 0.  M = D / omega
// (Jacobi).  Stopping test ||r||_2 / ||b||_2 < eps.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so the FP64 instruction count per
// row, not only the bytes, bounds these kernels.  The Jacobi scaling of the two
// products A M^-1 p and A M^-1 s is folded into a column-scaled copy of the
// matrix, a_ij / m_jj, built once per solve (one FMA per entry and right-hand
// side instead of a multiply and an FMA, and no gather of the diagonal), and
// x += alpha M^-1 p + omega M^-1 s is taken as x += M^-1 (alpha p + omega s).
// Both are the same iterates in exact arithmetic; the rounding differs from the
// unfolded form by a unit in the last place per product.
#include "krylov_dev.cuh"

#include <algorithm>
#include <cmath>

namespace sysu {

std::atomic<long> g_launches{0};

SellPattern make_sell(int n, const std::vector<int> &row_ptr, const std::vector<int> &cols) {
    SellPattern p;
    p.n = n;
    p.nslices = (n + 31) / 32;
    p.sl_ptr.assign(p.nslices + 1, 0);
    p.sl_w.assign(p.nslices, 0);
    p.row_len.assign(n, 0);
    for (int i = 0; i < n; ++i) p.row_len[i] = row_ptr[i + 1] - row_ptr[i];
    long off = 0;
    for (int s = 0; s < p.nslices; ++s) {
        int w = 0;
        for (int i = s * 32; i < std::min(n, s * 32 + 32); ++i) w = std::max(w, p.row_len[i]);
        p.sl_w[s] = w;
        p.sl_ptr[s] = (int)off;
        off += (long)w * 32;
    }
    p.sl_ptr[p.nslices] = (int)off;
    p.nnz = off;
    p.nnz_true = row_ptr[n];
    p.col.assign(off, 0);
    for (int s = 0; s < p.nslices; ++s) {
        for (int lane = 0; lane < 32; ++lane) {
            int i = s * 32 + lane;
            int self = i < n ? i : (n - 1);
            for (int k = 0; k < p.sl_w[s]; ++k) {
                long e = (long)p.sl_ptr[s] + (long)k * 32 + lane;
                p.col[e] = (i < n && k < p.row_len[i]) ? cols[row_ptr[i] + k] : self;
            }
        }
    }
    return p;
}

void SellDev::upload(const SellPattern &p, cudaStream_t s) {
    n = p.n;
    nslices = p.nslices;
    wmax = 0;
    for (int w : p.sl_w) wmax = std::max(wmax, w);
    nnz = p.nnz;
    nnz_true = p.nnz_true;
    sl_ptr.upload(p.sl_ptr, s);
    sl_w.upload(p.sl_w, s);
    col.upload(p.col, s);
    // level schedule of the triangular sweeps (natural row order)
    std::vector<int> lf(p.n, 0), lb(p.n, 0);
    int nf = 0, nb = 0;
    for (int i = 0; i < p.n; ++i) {
        int l = 0;
        for (int k = 1; k < p.row_len[i]; ++k) {
            int j = p.col[p.pos(i, k)];
            if (j < i) l = std::max(l, lf[j] + 1);
        }
        lf[i] = l;
        nf = std::max(nf, l + 1);
    }
    for (int i = p.n - 1; i >= 0; --i) {
        int l = 0;
        for (int k = 1; k < p.row_len[i]; ++k) {
            int j = p.col[p.pos(i, k)];
            if (j > i) l = std::max(l, lb[j] + 1);
        }
        lb[i] = l;
        nb = std::max(nb, l + 1);
    }
    auto group = [&](const std::vector<int> &lv, int nl, std::vector<int> &ptr, std::vector<int> &rows) {
        ptr.assign(nl + 1, 0);
        for (int i = 0; i < p.n; ++i) ptr[lv[i] + 1]++;
        for (int l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
        rows.assign(p.n, 0);
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int i = 0; i < p.n; ++i) rows[fill[lv[i]]++] = i;
    };
    std::vector<int> fp, fr, bp, br;
    if (p.n > 0) {
        group(lf, nf, fp, fr);
        group(lb, nb, bp, br);
    }
    lev.nf = p.n > 0 ? nf : 0;
    lev.nb = p.n > 0 ? nb : 0;
    lev.fptr.upload(fp, s);
    lev.frows.upload(fr, s);
    lev.bptr.upload(bp, s);
    lev.brows.upload(br, s);
    auto info = [&](const std::vector<int> &rows) {
        std::vector<int4> v(rows.size());
        for (size_t r = 0; r < rows.size(); ++r) {
            int i = rows[r];
            v[r] = make_int4(i, p.sl_ptr[i >> 5] + (i & 31), p.sl_w[i >> 5], 0);
        }
        return v;
    };
    lev.finfo.upload(info(fr), s);
    lev.binfo.upload(info(br), s);
}

namespace {

// y_c = A (dinv .* x_c) for NR right-hand sides, skipping inactive ones, from
// the column-scaled values sv[e] = a_e dinv[col e].  MULTI: right-hand side c
// has its own scaled values svals[c] (same pattern); the column indices are
// read once.
template <int NR, bool MULTI>
__device__ __forceinline__ void row_dot_scaled(const SellView &A, const double *const *svals, int i,
                                               const double *__restrict__ x, int n, const bool (&act)[3],
                                               double (&y)[NR]) {
    int s = i >> 5;
    int e = A.sl_ptr[s] + (i & 31);
    int w = A.sl_w[s];
#pragma unroll
    for (int c = 0; c < NR; ++c) y[c] = 0.0;
    for (int k = 0; k < w; ++k, e += 32) {
        int j = A.col[e];
        if (MULTI) {
#pragma unroll
            for (int c = 0; c < NR; ++c)
                if (act[c]) y[c] = fma(svals[c][e], x[(size_t)c * n + j], y[c]);
        } else {
            double a = svals[0][e];
#pragma unroll
            for (int c = 0; c < NR; ++c)
                if (act[c]) y[c] = fma(a, x[(size_t)c * n + j], y[c]);
        }
    }
}

// sv[e] = val[e] dinv[col e] over all stored entries (padding entries hold 0
// and their own row as the column).
__global__ void k_scale_cols(long nnz, const int *__restrict__ col, const double *__restrict__ val,
                             const double *__restrict__ dinv, double *__restrict__ sv) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nnz) sv[e] = val[e] * dinv[col[e]];
}

__global__ void k_jacobi_apply(SellView A, double omega, const double *c, double *y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    double d = A.val[A.sl_ptr[i >> 5] + (i & 31)];
    y[i] = omega * c[i] / d;
}

// Standalone SELL-32 product for the SpMV sweep: one row per thread, a warp per
// slice; the matrix is streamed with evict-first loads (read once), all of a row's
// entries are loaded before its FMAs, x is gathered through the read-only path.
template <class V>
__global__ void __launch_bounds__(256) k_spmv_stream(int n, const int *__restrict__ sl_ptr,
                                                     const int *__restrict__ sl_w, const int *__restrict__ col,
                                                     const V *__restrict__ val, const V *__restrict__ x,
                                                     V *__restrict__ y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = i >> 5;
    int e = __ldg(sl_ptr + s) + (i & 31);
    int w = __ldg(sl_w + s);
    V acc = (V)0;
    if (w <= 8) {
        int c[8];
        V a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < w) {
                c[k] = __ldcs(col + e + 32 * k);
                a[k] = __ldcs(val + e + 32 * k);
            }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < w) acc = fma(a[k], __ldg(x + c[k]), acc);
    } else {
        for (int k = 0; k < w; ++k) acc = fma(__ldcs(val + e + 32 * k), __ldg(x + __ldcs(col + e + 32 * k)), acc);
    }
    y[i] = acc;
}

// The same product with x staged in shared memory: block b (rows r0 .. r0+255)
// first loads x[r0 - SPMV_HALO, r0 + 256 + SPMV_HALO) with coalesced loads, and
// every column inside that window is read from there, the rest from global
// memory.  On the tet and hex meshes most of a row's neighbours lie within a few
// rows of it (the cells of one hex, the next hex along x), so about half of the
// gathers become shared-memory reads of a tile fetched in one stream.  Same FMA
// order as k_spmv_stream: the same bits.
constexpr int SPMV_HALO = 96;
template <class V>
__global__ void __launch_bounds__(256) k_spmv_stage(int n, const int *__restrict__ sl_ptr,
                                                    const int *__restrict__ sl_w, const int *__restrict__ col,
                                                    const V *__restrict__ val, const V *__restrict__ x,
                                                    V *__restrict__ y) {
    __shared__ V xs[256 + 2 * SPMV_HALO];
    const int r0 = blockIdx.x * 256;
    const int lo = r0 - SPMV_HALO;
    for (int q = threadIdx.x; q < 256 + 2 * SPMV_HALO; q += 256) {
        const int j = lo + q;
        xs[q] = (j >= 0 && j < n) ? __ldg(x + j) : (V)0;
    }
    __syncthreads();
    const int i = r0 + threadIdx.x;
    if (i >= n) return;
    const int s = i >> 5;
    const int e = __ldg(sl_ptr + s) + (i & 31);
    const int w = __ldg(sl_w + s);
    V acc = (V)0;
    for (int k = 0; k < w; ++k) {
        const int c = __ldcs(col + e + 32 * k);
        const V a = __ldcs(val + e + 32 * k);
        const unsigned q = (unsigned)(c - lo);
        const V xv = q < (unsigned)(256 + 2 * SPMV_HALO) ? xs[q] : __ldg(x + c);
        acc = fma(a, xv, acc);
    }
    y[i] = acc;
}

// The same product with a persistent grid: each warp takes SPW slices at a time
// (slices s, s + W, ... for W warps in the grid), so every thread has SPW rows'
// matrix entries in flight before its first gather.
template <class V, int SPW>
__global__ void __launch_bounds__(256) k_spmv_multi(int n, int nslices, const int *__restrict__ sl_ptr,
                                                    const int *__restrict__ sl_w, const int *__restrict__ col,
                                                    const V *__restrict__ val, const V *__restrict__ x,
                                                    V *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int W = (gridDim.x * blockDim.x) >> 5;
    for (int s0 = warp; s0 < nslices; s0 += SPW * W) {
        int e[SPW], w[SPW];
#pragma unroll
        for (int q = 0; q < SPW; ++q) {
            int s = s0 + q * W;
            w[q] = 0;
            e[q] = 0;
            if (s < nslices) {
                e[q] = __ldg(sl_ptr + s) + lane;
                w[q] = __ldg(sl_w + s);
            }
        }
        int c[SPW][8];
        V a[SPW][8];
#pragma unroll
        for (int q = 0; q < SPW; ++q)
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < w[q]) {
                    c[q][k] = __ldcs(col + e[q] + 32 * k);
                    a[q][k] = __ldcs(val + e[q] + 32 * k);
                }
        V acc[SPW];
#pragma unroll
        for (int q = 0; q < SPW; ++q) {
            acc[q] = (V)0;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < w[q]) acc[q] = fma(a[q][k], __ldg(x + c[q][k]), acc[q]);
            for (int k = 8; k < w[q]; ++k)
                acc[q] = fma(__ldcs(val + e[q] + 32 * k), __ldg(x + __ldcs(col + e[q] + 32 * k)), acc[q]);
        }
#pragma unroll
        for (int q = 0; q < SPW; ++q) {
            int row = (s0 + q * W) * 32 + lane;
            if (w[q] > 0 && row < n) y[row] = acc[q];
        }
    }
}

// The same product with the matrix entries staged in shared memory by each warp
// through cp.async (4- and 8-byte copies, no registers held while they are in
// flight): a warp takes slices gw, gw + W, ... and keeps SPMV_AS of them in a
// pipeline -- the entries of the slice SPMV_AS - 1 ahead are copied while the
// current slice's x gathers and FMAs run, and the slice pointers are loaded one
// step before they are needed.  A thread reads back only the entries it copied
// itself, so cp.async.wait_group alone orders them.  Slices wider than
// SPMV_AW are read from global memory.  Same FMA order as k_spmv_stream.
constexpr int SPMV_AS = 3;    // slices in flight per warp
constexpr int SPMV_AW = 8;    // widest staged slice
constexpr int SPMV_AT = 256;  // threads per block

template <int B>
__device__ __forceinline__ void cp_async_ca(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src),
                 "n"(B)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <class V>
constexpr size_t spmv_async_smem() {
    return (size_t)(SPMV_AT / 32) * SPMV_AS * 32 * SPMV_AW * (sizeof(V) + sizeof(int));
}

template <class V>
__global__ void __launch_bounds__(SPMV_AT) k_spmv_async(int n, int nslices, const int *__restrict__ sl_ptr,
                                                        const int *__restrict__ sl_w, const int *__restrict__ col,
                                                        const V *__restrict__ val, const V *__restrict__ x,
                                                        V *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char spmv_smem[];
    constexpr int SLOT = 32 * SPMV_AW;  // entries of one stage
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * (SPMV_AT / 32) + wib;
    const int W = gridDim.x * (SPMV_AT / 32);
    V *vb = reinterpret_cast<V *>(spmv_smem) + (size_t)wib * SPMV_AS * SLOT;
    int *cb = reinterpret_cast<int *>(spmv_smem + (size_t)(SPMV_AT / 32) * SPMV_AS * SLOT * sizeof(V)) +
              (size_t)wib * SPMV_AS * SLOT;
    const int J = gw < nslices ? (nslices - 1 - gw) / W + 1 : 0;  // slices of this warp
    int me[SPMV_AS], mw[SPMV_AS];                                  // slice pointer and width, by stage
    auto load_meta = [&](int j, int &e, int &w) {
        e = 0;
        w = 0;
        if (j < J) {
            const int s = gw + j * W;
            e = __ldg(sl_ptr + s);
            w = __ldg(sl_w + s);
        }
    };
    auto issue = [&](int j, int stage, int e, int w) {
        if (j < J && w <= SPMV_AW) {
            const int eb = e + lane;
            V *vd = vb + stage * SLOT + lane;
            int *cd = cb + stage * SLOT + lane;
            for (int k = 0; k < w; ++k) {
                cp_async_ca<(int)sizeof(V)>(vd + 32 * k, val + eb + 32 * k);
                cp_async_ca<4>(cd + 32 * k, col + eb + 32 * k);
            }
        }
        cp_async_commit();  // possibly empty: one group per slice keeps the count uniform
    };
#pragma unroll
    for (int u = 0; u < SPMV_AS; ++u) load_meta(u, me[u], mw[u]);
#pragma unroll
    for (int u = 0; u < SPMV_AS - 1; ++u) issue(u, u, me[u], mw[u]);
    for (int j0 = 0; j0 < J; j0 += SPMV_AS) {
#pragma unroll
        for (int u = 0; u < SPMV_AS; ++u) {
            const int j = j0 + u;
            cp_async_wait<SPMV_AS - 2>();  // slice j's copies have landed
            if (j < J) {
                const int row = (gw + j * W) * 32 + lane;
                const int w = mw[u];
                V acc = (V)0;
                if (w <= SPMV_AW) {
                    int c[SPMV_AW];
                    V xv[SPMV_AW];
#pragma unroll
                    for (int k = 0; k < SPMV_AW; ++k)
                        if (k < w) c[k] = cb[u * SLOT + 32 * k + lane];
#pragma unroll
                    for (int k = 0; k < SPMV_AW; ++k)
                        if (k < w) xv[k] = __ldg(x + c[k]);
#pragma unroll
                    for (int k = 0; k < SPMV_AW; ++k)
                        if (k < w) acc = fma(vb[u * SLOT + 32 * k + lane], xv[k], acc);
                } else {
                    const int e = me[u] + lane;
                    for (int k = 0; k < w; ++k) acc = fma(__ldcs(val + e + 32 * k), __ldg(x + __ldcs(col + e + 32 * k)), acc);
                }
                if (row < n) y[row] = acc;
            }
            // the slice SPMV_AS - 1 ahead goes into the stage freed one step ago
            const int nxt = (u + SPMV_AS - 1) % SPMV_AS;
            issue(j + SPMV_AS - 1, nxt, me[nxt], mw[nxt]);
            load_meta(j + SPMV_AS, me[u], mw[u]);
        }
    }
    cp_async_wait<0>();
}

int g_spmv_variant = 0;

// Reads a buffer larger than L2 (16-byte loads, one word written) so the
// caches hold clean lines of it: evicting them costs no write-back, unlike a
// flush by writes, whose dirty lines would be written back during the next
// kernel and inflate its DRAM traffic.
__global__ void k_l2_flush_read(const uint4 *__restrict__ buf, size_t n16, unsigned *sink) {
    unsigned acc = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x) {
        uint4 v = __ldcg(buf + i);
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    if (acc == 0x9e3779b9u) *sink = acc;  // keeps the loads; practically never taken
}

// A fixed, non-trivial x for the SpMV sweep: 1 + hash(i) / 2000.
__global__ void k_fill_x(long n, double *x64, float *x32) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = 1.0 + 0.5 * (double)((i * 2654435761ull) % 1000) / 1000.0;
    x64[i] = v;
    x32[i] = (float)v;
}

// sv[e] = (float)(val[e] dinv[col e]) over all stored entries
__global__ void k_scale_cols32(long nnz, const int *__restrict__ col, const double *__restrict__ val,
                               const double *__restrict__ dinv, float *__restrict__ sv) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nnz) sv[e] = (float)(val[e] * dinv[col[e]]);
}

__global__ void k_to_fp32(long n, const double *src, float *dst) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}


struct BicgArgs {
    SellView A;
    const double *vals[3];  // per right-hand-side matrix values (MULTI)
    const double *svals[3]; // the same, column-scaled by the Jacobi diagonal inverse
    const double *b[3];
    double *x[3];
    double *r, *rt, *p, *v, *s, *t;
    const double *dinv;
    double *partials;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit;
    double eps;
    // behind a mixed solve: run only if gate->status[0] is DEV_STALLED (one
    // system; the iterations of both are reported); null: always run
    const SolveInfo *gate;
};

// Scalar state of a BiCGSTAB solve.  Thread 0 of every block derives it from
// the global sums (which every block adds up in the same fixed order, so all
// blocks hold identical copies) and the block reads it from shared memory:
// the square roots and divisions run once per block instead of in every thread,
// and the vector loops keep only the few scalars they use in registers.
struct BicgState {
    double bnorm[3], res[3], rho[3], rho_prev[3], alpha[3], omg[3], beta[3], snorm[3];
    int it[3], status[3], done[3], act[3], early[3], act2[3];
    int any;
};

template <int NR, bool MULTI>
__global__ void __launch_bounds__(KB, 4) k_bicgstab(BicgArgs a) {
    if (a.gate && a.gate->status[0] != DEV_STALLED) return;  // the same word for every block
    const int it_before = a.gate ? a.gate->iters[0] : 0;
    const int n = a.A.n;
    const int T = gridDim.x * KB;
    const int t0 = blockIdx.x * KB + threadIdx.x;
    const bool lead = threadIdx.x == 0;
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const double *__restrict__ dinv = a.dinv;
    const size_t N = (size_t)n;
    __shared__ BicgState S;
    {
        double v[2 * NR];
#pragma unroll
        for (int c = 0; c < 2 * NR; ++c) v[c] = 0.0;
        for (int i = t0; i < n; i += T) {
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                double bi = a.b[c][i];
                SellView Ac = a.A;
                if (MULTI) Ac.val = a.vals[c];
                double ri = bi - row_dot(Ac, i, a.x[c]);
                a.r[c * N + i] = ri;
                a.rt[c * N + i] = ri;
                v[c] += bi * bi;
                v[NR + c] += ri * ri;
            }
        }
        if (!grid_reduce_t0<2 * NR>(v, rc, a.gb, err)) return;
        if (lead) {
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                double bn = sqrt(v[c]);
                if (bn == 0.0) bn = 1.0;
                S.bnorm[c] = bn;
                S.res[c] = sqrt(v[NR + c]) / bn;
                S.rho[c] = v[NR + c];
                S.rho_prev[c] = S.alpha[c] = S.omg[c] = 1.0;
                S.it[c] = 0;
                S.status[c] = DEV_OK;
                S.done[c] = 0;
            }
        }
    }
    bool act[3] = {false, false, false};
    for (;;) {
        if (lead) {
            int any = 0;
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                bool ac = !S.done[c] && !(S.res[c] < a.eps) && S.it[c] < a.maxit;
                if (ac && !isfinite(S.res[c])) { S.done[c] = 1; S.status[c] = DEV_NONFINITE; ac = false; }
                if (ac && S.rho[c] == 0.0) { S.done[c] = 1; S.status[c] = DEV_BREAKDOWN; ac = false; }
                if (ac) {
                    ++S.it[c];
                    any = 1;
                    S.beta[c] = (S.it[c] == 1) ? 0.0 : (S.rho[c] / S.rho_prev[c]) * (S.alpha[c] / S.omg[c]);
                }
                S.act[c] = ac;
            }
            S.any = any;
        }
        __syncthreads();
        if (!S.any) break;
        // p = r + beta (p - omega v)
        {
            double beta[NR], omg[NR];
            bool first[NR];
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                act[c] = S.act[c] != 0;
                beta[c] = S.beta[c];
                omg[c] = S.omg[c];
                first[c] = S.it[c] == 1;
            }
            for (int i = t0; i < n; i += T) {
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act[c]) continue;
                    size_t k = c * N + i;
                    a.p[k] = first[c] ? a.r[k] : a.r[k] + beta[c] * (a.p[k] - omg[c] * a.v[k]);
                }
            }
        }
        if (!grid_sync(a.gb, err)) return;
        // v = A M^-1 p ; rt . v
        {
            double red[NR];
#pragma unroll
            for (int c = 0; c < NR; ++c) red[c] = 0.0;
            for (int i = t0; i < n; i += T) {
                double y[NR];
                row_dot_scaled<NR, MULTI>(a.A, a.svals, i, a.p, n, act, y);
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act[c]) continue;
                    a.v[c * N + i] = y[c];
                    red[c] += a.rt[c * N + i] * y[c];
                }
            }
            if (!grid_reduce_t0<NR>(red, rc, a.gb, err)) return;
            if (lead) {
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!S.act[c]) continue;
                    if (red[c] == 0.0) { S.done[c] = 1; S.status[c] = DEV_BREAKDOWN; S.act[c] = 0; continue; }
                    S.alpha[c] = S.rho[c] / red[c];
                }
            }
            __syncthreads();
        }
        // s = r - alpha v ; ||s||
        {
            double red[NR], alpha[NR];
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                red[c] = 0.0;
                act[c] = S.act[c] != 0;
                alpha[c] = S.alpha[c];
            }
            for (int i = t0; i < n; i += T) {
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act[c]) continue;
                    size_t k = c * N + i;
                    double si = a.r[k] - alpha[c] * a.v[k];
                    a.s[k] = si;
                    red[c] += si * si;
                }
            }
            if (!grid_reduce_t0<NR>(red, rc, a.gb, err)) return;
            if (lead) {
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    S.early[c] = 0;
                    S.act2[c] = 0;
                    if (!S.act[c]) continue;
                    S.snorm[c] = sqrt(red[c]) / S.bnorm[c];
                    S.early[c] = S.snorm[c] < a.eps;
                    S.act2[c] = !S.early[c];
                }
            }
            __syncthreads();
        }
        // t = A M^-1 s ; t.s, t.t
        {
            bool act2[3] = {false, false, false};
#pragma unroll
            for (int c = 0; c < NR; ++c) act2[c] = S.act2[c] != 0;
            double red[2 * NR];
#pragma unroll
            for (int c = 0; c < 2 * NR; ++c) red[c] = 0.0;
            for (int i = t0; i < n; i += T) {
                double y[NR];
                row_dot_scaled<NR, MULTI>(a.A, a.svals, i, a.s, n, act2, y);
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act2[c]) continue;
                    size_t k = c * N + i;
                    a.t[k] = y[c];
                    red[c] += y[c] * a.s[k];
                    red[NR + c] += y[c] * y[c];
                }
            }
            if (!grid_reduce_t0<2 * NR>(red, rc, a.gb, err)) return;
            if (lead) {
#pragma unroll
                for (int c = 0; c < NR; ++c)
                    if (S.act2[c]) S.omg[c] = red[NR + c] != 0.0 ? red[c] / red[NR + c] : 0.0;
            }
            __syncthreads();
        }
        // x += M^-1 (alpha p + omega s) ; r = s - omega t
        {
            double red[2 * NR], alpha[NR], omg[NR];
            bool early[NR];
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                red[c] = red[NR + c] = 0.0;
                alpha[c] = S.alpha[c];
                omg[c] = S.omg[c];
                early[c] = S.early[c] != 0;
            }
            for (int i = t0; i < n; i += T) {
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act[c]) continue;
                    size_t k = c * N + i;
                    double di = MULTI ? dinv[k] : dinv[i];
                    if (early[c]) {
                        a.x[c][i] += alpha[c] * (di * a.p[k]);
                    } else {
                        double si = a.s[k];
                        a.x[c][i] = fma(di, fma(alpha[c], a.p[k], omg[c] * si), a.x[c][i]);
                        double ri = fma(-omg[c], a.t[k], si);
                        a.r[k] = ri;
                        red[c] += ri * ri;
                        red[NR + c] += a.rt[k] * ri;
                    }
                }
            }
            if (!grid_reduce_t0<2 * NR>(red, rc, a.gb, err)) return;
            if (lead) {
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!S.act[c]) continue;
                    if (S.early[c]) {
                        S.res[c] = S.snorm[c];
                        S.done[c] = 1;
                    } else {
                        S.res[c] = sqrt(red[c]) / S.bnorm[c];
                        S.rho_prev[c] = S.rho[c];
                        S.rho[c] = red[NR + c];
                        if (S.omg[c] == 0.0 && !(S.res[c] < a.eps)) { S.done[c] = 1; S.status[c] = DEV_BREAKDOWN; }
                    }
                }
            }
        }
    }
    if (blockIdx.x == 0 && lead) {
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            int st = S.status[c];
            if (st == DEV_OK && !(S.res[c] < a.eps)) st = isfinite(S.res[c]) ? DEV_MAXITER : DEV_NONFINITE;
            a.info->status[c] = st;
            a.info->iters[c] = S.it[c] + (c == 0 ? it_before : 0);
            a.info->res[c] = S.res[c];
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed-precision BiCGSTAB for one system: FP32 inner iterations on the
// correction equation A e = r, FP64 defect correction.  The FP32 vectors hold
// the residual scaled by a power of two sig with sig ||r|| ~ 1 (pow2_scale),
// so residuals that have become tiny in FP64 do not underflow in FP32.  The inner recurrences
// are those of k_bicgstab with FP32 vectors and the column-scaled FP32 matrix
// a_ij / m_jj (rounded from FP64); its dot products are FP32 over a thread's
// rows and summed across threads in FP64.  Once the FP32 residual has fallen
// by inner_tol since the last update (or s is that small already, or a
// recurrence breaks down), x += M^-1 e in FP64, the FP64 residual b - A x
// replaces r and the inner process restarts from it.  Convergence is decided
// on that FP64 residual only: ||b - A x|| / ||b|| < eps, the test of the FP64
// solve.  Three updates in a row that do not lower the FP64 residual end it
// with DEV_STALLED, and the FP64 BiCGSTAB launched behind it continues from x.  info->iters counts inner iterations,
// info->refinements the FP64 updates.
struct BicgMixedArgs {
    SellView A;            // FP64 values (residuals)
    const float *sv32;     // FP32 column-scaled values
    const double *b;
    double *x;
    const double *dinv;    // FP64 Jacobi diagonal inverse
    double *r64;           // FP64 residual scratch
    float *r, *rt, *p, *v, *s, *t, *e;  // in units of sig (a power of two, sig ||r|| ~ 1)
    double *partials;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit;
    double eps, inner_tol;
};

struct BicgMixedState {
    double bb, thr, rr64, rr_ref, r0in, rho, rho_prev, alpha, omg, beta, snorm2, sig;
    int it, inner, status, upd, stall, act, early, done;
};

// y = A_s x over FP32 column-scaled values, one row (FMA order of row_dot_scaled)
__device__ __forceinline__ float row_dot32(const SellView &A, const float *__restrict__ sv, int i,
                                           const float *__restrict__ x) {
    const int s = i >> 5;
    int e = A.sl_ptr[s] + (i & 31);
    const int w = A.sl_w[s];
    float y = 0.f;
    for (int k = 0; k < w; ++k, e += 32) y = fmaf(sv[e], x[A.col[e]], y);
    return y;
}

__global__ void __launch_bounds__(KB, 4) k_bicgstab_mixed(BicgMixedArgs a) {
    const int n = a.A.n;
    const int T = gridDim.x * KB;
    const int t0 = blockIdx.x * KB + threadIdx.x;
    const bool lead = threadIdx.x == 0;
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    __shared__ BicgMixedState S;
    // FP64 residual of x into r (FP32), rt = r, e = p = v = 0; ||b||^2 (first
    // call) and ||b - A x||^2.  The lead thread then restarts the inner process.
    auto residual = [&](bool first) -> bool {
        double v2[2] = {0.0, 0.0}, rf2 = 0.0;
        for (int i = t0; i < n; i += T) {
            const double bi = a.b[i];
            const double ri = bi - row_dot(a.A, i, a.x);
            a.r64[i] = ri;
            if (first) v2[0] = fma(bi, bi, v2[0]);
            v2[1] = fma(ri, ri, v2[1]);
        }
        if (!grid_reduce_t0<2>(v2, rc, a.gb, err)) return false;
        if (lead) S.sig = pow2_scale(v2[1]);  // the FP32 vectors hold sig r (exact scaling)
        __syncthreads();
        {
            const double sg = S.sig;
            float f2 = 0.f;
            for (int i = t0; i < n; i += T) {
                const float rf = (float)(sg * a.r64[i]);
                a.r[i] = rf;
                a.rt[i] = rf;
                a.e[i] = 0.f;
                a.p[i] = 0.f;
                a.v[i] = 0.f;
                f2 = fmaf(rf, rf, f2);
            }
            double v1[1] = {(double)f2};
            if (!grid_reduce_t0<1>(v1, rc, a.gb, err)) return false;
            rf2 = v1[0];
        }
        if (lead) {
            if (first) {
                S.bb = v2[0] == 0.0 ? 1.0 : v2[0];
                S.thr = a.eps * a.eps * S.bb;
                S.it = 0;
                S.upd = 0;
                S.stall = 0;
                S.status = DEV_OK;
                S.done = 0;
                S.rr_ref = v2[1];
            } else {
                ++S.upd;
                S.stall = v2[1] < S.rr_ref ? 0 : S.stall + 1;
                S.rr_ref = fmin(S.rr_ref, v2[1]);
            }
            S.rr64 = v2[1];
            S.r0in = rf2;
            S.rho = rf2;  // rt . r with rt = r, in the FP32 inner precision (sig^2 units)
            S.rho_prev = S.alpha = S.omg = 1.0;
            S.inner = 0;
            if (!isfinite(v2[1])) { S.status = DEV_NONFINITE; S.done = 1; }
            else if (v2[1] < S.thr) S.done = 1;
            else if (S.stall >= 3) { S.status = DEV_STALLED; S.done = 1; }  // FP64 takes over
            else if (S.it >= a.maxit) { S.status = DEV_MAXITER; S.done = 1; }
        }
        __syncthreads();
        return true;
    };
    // x += M^-1 e / sig in FP64, then the FP64 residual
    auto update = [&]() -> bool {
        const double isg = 1.0 / S.sig;
        for (int i = t0; i < n; i += T) a.x[i] = fma(a.dinv[i] * isg, (double)a.e[i], a.x[i]);
        if (!grid_sync(a.gb, err)) return false;
        return residual(false);
    };
    if (!residual(true)) return;
    const float *__restrict__ sv = a.sv32;
    const double d2 = a.inner_tol * a.inner_tol;
    for (;;) {
        if (S.done) break;
        // p = r + beta (p - omega v)
        if (lead) {
            ++S.it;
            ++S.inner;
            S.beta = S.inner == 1 ? 0.0 : (S.rho / S.rho_prev) * (S.alpha / S.omg);
        }
        __syncthreads();
        {
            const float beta = (float)S.beta, omg = (float)S.omg;
            const bool first = S.inner == 1;
            for (int i = t0; i < n; i += T)
                a.p[i] = first ? a.r[i] : fmaf(beta, fmaf(-omg, a.v[i], a.p[i]), a.r[i]);
        }
        if (!grid_sync(a.gb, err)) return;
        // v = A M^-1 p ; rt . v
        {
            float f = 0.f;
            for (int i = t0; i < n; i += T) {
                const float y = row_dot32(a.A, sv, i, a.p);
                a.v[i] = y;
                f = fmaf(a.rt[i], y, f);
            }
            double red[1] = {(double)f};
            if (!grid_reduce_t0<1>(red, rc, a.gb, err)) return;
            if (lead) {
                S.act = red[0] != 0.0;  // 0: the recurrence broke down, update and restart
                if (S.act) S.alpha = S.rho / red[0];
            }
            __syncthreads();
        }
        if (!S.act) {
            if (!update()) return;
            continue;
        }
        // s = r - alpha v ; ||s||
        {
            const float alpha = (float)S.alpha;
            float f = 0.f;
            for (int i = t0; i < n; i += T) {
                const float si = fmaf(-alpha, a.v[i], a.r[i]);
                a.s[i] = si;
                f = fmaf(si, si, f);
            }
            double red[1] = {(double)f};
            if (!grid_reduce_t0<1>(red, rc, a.gb, err)) return;
            if (lead) {
                S.snorm2 = red[0];
                S.early = red[0] <= d2 * S.r0in;
            }
            __syncthreads();
        }
        if (S.early) {  // e += alpha p, then the FP64 update
            const float alpha = (float)S.alpha;
            for (int i = t0; i < n; i += T) a.e[i] = fmaf(alpha, a.p[i], a.e[i]);
            if (!update()) return;
            continue;
        }
        // t = A M^-1 s ; t.s, t.t
        {
            float f0 = 0.f, f1 = 0.f;
            for (int i = t0; i < n; i += T) {
                const float y = row_dot32(a.A, sv, i, a.s);
                a.t[i] = y;
                f0 = fmaf(y, a.s[i], f0);
                f1 = fmaf(y, y, f1);
            }
            double red[2] = {(double)f0, (double)f1};
            if (!grid_reduce_t0<2>(red, rc, a.gb, err)) return;
            if (lead) S.omg = red[1] != 0.0 ? red[0] / red[1] : 0.0;
            __syncthreads();
        }
        // e += alpha p + omega s ; r = s - omega t ; r.r, rt.r
        {
            const float alpha = (float)S.alpha, omg = (float)S.omg;
            float f0 = 0.f, f1 = 0.f;
            for (int i = t0; i < n; i += T) {
                const float si = a.s[i];
                a.e[i] = fmaf(alpha, a.p[i], fmaf(omg, si, a.e[i]));
                const float ri = fmaf(-omg, a.t[i], si);
                a.r[i] = ri;
                f0 = fmaf(ri, ri, f0);
                f1 = fmaf(a.rt[i], ri, f1);
            }
            double red[2] = {(double)f0, (double)f1};
            if (!grid_reduce_t0<2>(red, rc, a.gb, err)) return;
            if (lead) {
                S.rho_prev = S.rho;
                S.rho = red[1];
                // FP64 update once the FP32 residual fell by inner_tol, at the
                // iteration cap, or when the next step would divide by zero
                S.act = !(red[0] <= d2 * S.r0in || S.it >= a.maxit || S.omg == 0.0 || S.rho == 0.0 ||
                          !(red[0] == red[0]));
            }
            __syncthreads();
        }
        if (!S.act && !update()) return;
    }
    if (blockIdx.x == 0 && lead) {
        a.info->status[0] = S.status;
        a.info->iters[0] = S.it;
        a.info->res[0] = sqrt(S.rr64) / sqrt(S.bb);
        a.info->refinements = S.upd;
    }
}

}  // namespace

void KrylovWork::ensure(int n_, int nrhs_, int max_blocks_, cudaStream_t st) {
    if (n_ <= n && nrhs_ <= nrhs && max_blocks_ <= max_blocks) return;
    n = std::max(n, n_);
    nrhs = std::max(nrhs, nrhs_);
    max_blocks = std::max(max_blocks, max_blocks_);
    size_t m = (size_t)n * nrhs;
    r.alloc(m); rt.alloc(m); p.alloc(m); v.alloc(m); s.alloc(m); t.alloc(m);
    dinv.alloc(m);
    partials.alloc((size_t)8 * NVMAX * max_blocks);  // also the 4-word exact-sum partials
    barrier.alloc(1);
    barrier.zero(st);
}

void KrylovWork::ensure32(int n_, cudaStream_t st) {
    if (r32.size() >= (size_t)n_) return;
    r32.alloc(n_); z32.alloc(n_); p32.alloc(n_); q32.alloc(n_); e32.alloc(n_); dinv32.alloc(n_);
    (void)st;
}

void sell_to_fp32(const SellDev &A, const double *val, float *val32, cudaStream_t st) {
    if (A.nnz == 0) return;
    { k_to_fp32<<<(unsigned)((A.nnz + KB - 1) / KB), KB, 0, st>>>(A.nnz, val, val32); ++::sysu::g_launches; }
    SYSU_CUDA(cudaGetLastError());
}


void spmv(const SellDev &A, const double *val, const double *x, double *y, cudaStream_t st) { spmv_stream(A, val, x, y, st); }

void fill_sweep_x(long n, double *x64, float *x32, cudaStream_t st) {
    if (n == 0) return;
    { k_fill_x<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x64, x32); ++::sysu::g_launches; }
    SYSU_CUDA(cudaGetLastError());
}

template <class V>
static void spmv_dispatch(const SellDev &A, const V *val, const V *x, V *y, cudaStream_t st) {
    if (A.n == 0) return;
    const int v = g_spmv_variant;
    if (v == SPMV_ASYNC) {
        static int per_sm[2] = {0, 0};
        int &ps = per_sm[sizeof(V) == 8 ? 1 : 0];
        const int sm = (int)spmv_async_smem<V>();
        if (!ps) {
            SYSU_CUDA(cudaFuncSetAttribute(k_spmv_async<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
            SYSU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, k_spmv_async<V>, SPMV_AT, sm));
            ps = std::max(ps, 1);
        }
        const int G = std::max(1, std::min((A.nslices + SPMV_AT / 32 - 1) / (SPMV_AT / 32), num_sms() * ps));
        k_spmv_async<V><<<G, SPMV_AT, sm, st>>>(A.n, A.nslices, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val, x, y);
    } else if (v == SPMV_STAGE) {
        k_spmv_stage<V><<<(A.n + 255) / 256, 256, 0, st>>>(A.n, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val, x, y);
    } else if (v == 0 || v == SPMV_RING) {
        k_spmv_stream<V><<<(A.n + 255) / 256, 256, 0, st>>>(A.n, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val, x, y);
    } else {
        int per_sm = v >= 10 ? v / 10 : 8;   // blocks of 256 per SM
        int spw = v % 10;
        int G = std::max(1, std::min((A.nslices * 32 + 255) / 256, num_sms() * per_sm));
        if (spw == 1)
            k_spmv_multi<V, 1><<<G, 256, 0, st>>>(A.n, A.nslices, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val, x, y);
        else if (spw == 2)
            k_spmv_multi<V, 2><<<G, 256, 0, st>>>(A.n, A.nslices, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val, x, y);
        else
            k_spmv_multi<V, 4><<<G, 256, 0, st>>>(A.n, A.nslices, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val, x, y);
    }
    ++::sysu::g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void spmv_stream(const SellDev &A, const double *val, const double *x, double *y, cudaStream_t st) {
    spmv_dispatch<double>(A, val, x, y, st);
}

void spmv_stream32(const SellDev &A, const float *val, const float *x, float *y, cudaStream_t st) {
    spmv_dispatch<float>(A, val, x, y, st);
}

void set_spmv_variant(int v) { g_spmv_variant = v; }
int spmv_variant() { return g_spmv_variant; }

void l2_flush_read(const void *buf, size_t bytes, unsigned *sink, cudaStream_t st) {
    size_t n16 = bytes / 16;
    if (!n16) return;
    { k_l2_flush_read<<<num_sms() * 8, 256, 0, st>>>(static_cast<const uint4 *>(buf), n16, sink); ++::sysu::g_launches; }
    SYSU_CUDA(cudaGetLastError());
}

void jacobi_apply(const SellDev &A, const double *val, double omega, const double *c, double *y, cudaStream_t st) {
    if (A.n == 0) return;
    { k_jacobi_apply<<<(A.n + KB - 1) / KB, KB, 0, st>>>(view(A, val), omega, c, y); ++::sysu::g_launches; }
    SYSU_CUDA(cudaGetLastError());
}


// Blocks of a BiCGSTAB launch: enough for about BICG_ROWS_PER_THREAD rows a
// thread, at least one per SM.  Each iteration has five grid barriers; on a
// small system (256k rows: 608 blocks would give under 2 rows a thread) the
// barriers of a full grid cost more than its extra parallelism brings -- the
// momentum solve of the 307k-cell channel measured 3.1 ms on 608 blocks and
// 2.3 ms on 256.  The 2M-row case keeps the full grid.
constexpr int BICG_ROWS_PER_THREAD = 4;
static int bicg_blocks_for(int n, int maxb) {
    const long want = ((long)n + (long)KB * BICG_ROWS_PER_THREAD - 1) / ((long)KB * BICG_ROWS_PER_THREAD);
    return (int)std::min<long>(maxb, std::max<long>(num_sms(), want));
}

static int bicg_max_blocks(int nrhs, bool multi) {
    static int mb[4] = {0, 0, 0, 0};
    if (!mb[0]) {
        mb[0] = coresident_blocks(k_bicgstab<1, false>);
        mb[1] = coresident_blocks(k_bicgstab<3, false>);
        mb[2] = coresident_blocks(k_bicgstab<3, true>);
        mb[3] = std::max(std::max(mb[0], mb[1]), mb[2]);
    }
    if (nrhs < 0) return mb[3];
    return nrhs == 1 ? mb[0] : (multi ? mb[2] : mb[1]);
}

static void bicg_launch(const SellDev &A, const double *const *vals, bool multi, int nrhs, const double *const *b,
                        double *const *x, const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st,
                        const SolveInfo *gate = nullptr) {
    int n = A.n;
    int maxb = bicg_max_blocks(nrhs, multi);
    if (w.sm_cap > 0) maxb = std::min(maxb, w.sm_cap * std::max(1, maxb / num_sms()));
    w.ensure(n, nrhs == 1 ? 1 : 3, bicg_max_blocks(-1, false), st);
    const int nmat = multi ? nrhs : 1;
    if (w.sval.size() < (size_t)A.nnz * nmat) w.sval.alloc((size_t)A.nnz * nmat);
    for (int c = 0; c < nmat; ++c) {
        SellView Vc = view(A, vals[c]);
        double *dc = w.dinv.get() + (size_t)c * n;
        { k_jacobi_dinv<<<(n + KB - 1) / KB, KB, 0, st>>>(Vc, o.omega, o.jacobi ? 1 : 0, dc); ++::sysu::g_launches; }
        if (A.nnz > 0) {
            k_scale_cols<<<(unsigned)((A.nnz + KB - 1) / KB), KB, 0, st>>>(A.nnz, A.col.get(), vals[c], dc,
                                                                          w.sval.get() + (size_t)c * A.nnz);
            ++::sysu::g_launches;
        }
    }
    if (!gate) SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    BicgArgs a{};
    a.gate = gate;
    a.A = view(A, vals[0]);
    for (int c = 0; c < 3; ++c) {
        a.vals[c] = vals[multi ? std::min(c, nrhs - 1) : 0];
        a.svals[c] = w.sval.get() + (size_t)(multi ? std::min(c, nrhs - 1) : 0) * A.nnz;
        a.b[c] = b[std::min(c, nrhs - 1)];
        a.x[c] = x[std::min(c, nrhs - 1)];
    }
    a.r = w.r.get(); a.rt = w.rt.get(); a.p = w.p.get(); a.v = w.v.get(); a.s = w.s.get(); a.t = w.t.get();
    a.dinv = w.dinv.get();
    a.partials = w.partials.get();
    a.gb = w.barrier.get();
    a.info = info;
    a.maxit = o.maxit;
    a.eps = o.eps;
    void *args[] = {&a};
    int G = grid_for(n, bicg_blocks_for(n, maxb));
    const void *k = nrhs == 1 ? (const void *)k_bicgstab<1, false>
                              : (multi ? (const void *)k_bicgstab<3, true> : (const void *)k_bicgstab<3, false>);
    SYSU_CUDA(cudaMemsetAsync(w.barrier.get(), 0, sizeof(GridBarrier), st));  // grid_sync starts from 0
    SYSU_CUDA(cudaLaunchCooperativeKernel(k, dim3(G), dim3(KB), args, 0, st));
    ++::sysu::g_launches;
}

void bicgstab_prepare(const SellDev &A, int nrhs, KrylovWork &w, cudaStream_t st) {
    if (A.n == 0) return;
    w.ensure(A.n, nrhs == 1 ? 1 : 3, bicg_max_blocks(-1, false), st);
    if (w.sval.size() < (size_t)A.nnz) w.sval.alloc(A.nnz);
}

void bicgstab_solve(const SellDev &A, const double *val, int nrhs, const double *const *b, double *const *x,
                    const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    if (A.n == 0) return;
    if (nrhs != 1 && nrhs != 3) throw CaseError{"bicgstab_solve: use 1 or 3 right-hand sides"};
    const double *vals[1] = {val};
    bicg_launch(A, vals, false, nrhs, b, x, o, w, info, st);
}

void bicgstab_solve_mixed(const SellDev &A, const double *val, const double *b, double *x, const KrylovOpts &o,
                          KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    const int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = coresident_blocks(k_bicgstab_mixed);
    int mb = maxb;
    if (w.sm_cap > 0) mb = std::min(mb, w.sm_cap * std::max(1, maxb / num_sms()));
    w.ensure(n, 1, std::max(bicg_max_blocks(-1, false), maxb), st);
    w.ensure32(n, st);
    if (w.rt32.size() < (size_t)n) {
        w.rt32.alloc(n); w.v32.alloc(n); w.s32.alloc(n); w.t32.alloc(n);
    }
    if (w.sval32.size() < (size_t)A.nnz) w.sval32.alloc(A.nnz);
    SellView V = view(A, val);
    { k_jacobi_dinv<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, o.jacobi ? 1 : 0, w.dinv.get()); ++::sysu::g_launches; }
    if (A.nnz > 0) {
        k_scale_cols32<<<(unsigned)((A.nnz + KB - 1) / KB), KB, 0, st>>>(A.nnz, A.col.get(), val, w.dinv.get(),
                                                                        w.sval32.get());
        ++::sysu::g_launches;
    }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    BicgMixedArgs a{};
    a.A = V;
    a.sv32 = w.sval32.get();
    a.b = b;
    a.x = x;
    a.dinv = w.dinv.get();
    a.r64 = w.r.get();
    a.r = w.r32.get(); a.rt = w.rt32.get(); a.p = w.p32.get(); a.v = w.v32.get();
    a.s = w.s32.get(); a.t = w.t32.get(); a.e = w.e32.get();
    a.partials = w.partials.get();
    a.gb = w.barrier.get();
    a.info = info;
    a.maxit = o.maxit;
    a.eps = o.eps;
    a.inner_tol = o.inner_tol;
    void *args[] = {&a};
    const int G = grid_for(n, bicg_blocks_for(n, mb));
    SYSU_CUDA(cudaMemsetAsync(w.barrier.get(), 0, sizeof(GridBarrier), st));  // grid_sync starts from 0
    SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_bicgstab_mixed, dim3(G), dim3(KB), args, 0, st));
    ++::sysu::g_launches;
    // FP64 takes over from the current x if the FP32 refinement stalled (the
    // launch returns at once otherwise)
    const double *bb[1] = {b};
    double *xx[1] = {x};
    const double *vv[1] = {val};
    bicg_launch(A, vv, false, 1, bb, xx, o, w, info, st, info);
}

void bicgstab_solve_multi(const SellDev &A, const double *const *vals, const double *const *b, double *const *x,
                          const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    if (A.n == 0) return;
    bicg_launch(A, vals, true, 3, b, x, o, w, info, st);
}

}  // namespace sysu
