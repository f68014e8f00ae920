// Persistent cooperative Krylov solvers on SELL-32 matrices (FP64).
//
// One solve = one cooperative launch.  Rows are distributed thread-per-row with
// a grid stride that is a multiple of 32, so each warp owns whole slices.
// Global dot products are reduced deterministically: warp shuffles, then the
// block, then every block sums the per-block partials in the same fixed order,
// so all blocks take identical convergence decisions and repeated runs are
// bit-identical.  Every barrier wait is bounded (device.hpp).
//
// Algorithms (restated from Barrett et al., "Templates", Figs. 2.5 and 2.10;
// they are the same recurrences as the CPU oracle's LASPack restatement):
//   CG        z = M^-1 r, rho = r.z, p = z + beta p, q = A p, alpha = rho/(p.q)
//   BiCGSTAB  right preconditioned, early exit on ||s||, breakdown on rho = 0
// M = D / omega (Jacobi).  Stopping test ||r||_2 / ||b||_2 < eps.
#include "krylov.hpp"

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
    nnz = p.nnz;
    nnz_true = p.nnz_true;
    sl_ptr.upload(p.sl_ptr, s);
    sl_w.upload(p.sl_w, s);
    col.upload(p.col, s);
}

namespace {

constexpr int KB = 256;
constexpr int NVMAX = 6;

struct RedCtx {
    double *partials;
    int G;
    int parity;
};

__device__ __shared__ double g_red_smem[NVMAX * 32];  // up to 32 warps per block
__device__ __shared__ double g_red_res[NVMAX];

// Block-reduce NV values, publish per-block partials, barrier, and give every
// thread the NV global sums.  Partials alternate between two buffers so that a
// block that runs ahead to the next reduction cannot overwrite values another
// block is still reading.
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], RedCtx &rc, GridBarrier *gb, int *err) {
    block_sum<NV>(v, g_red_smem);
    double *buf = rc.partials + (size_t)rc.parity * NVMAX * rc.G;
    rc.parity ^= 1;
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) buf[(size_t)k * rc.G + blockIdx.x] = v[k];
    if (!grid_sync(gb, err)) return false;
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = warp_sum_partials(buf + (size_t)k * rc.G, rc.G);
            if (threadIdx.x == 0) g_red_res[k] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = g_red_res[k];
    __syncthreads();
    return true;
}

// As grid_reduce, but the global sums are valid in thread 0 only: the caller
// derives its scalars there once per block and broadcasts them (divisions and
// square roots are long FP64 sequences; doing them in every thread costs more
// FP64 issue slots than a row of the vector updates).
template <int NV>
__device__ __forceinline__ bool grid_reduce_t0(double (&v)[NV], RedCtx &rc, GridBarrier *gb, int *err) {
    block_sum_t0<NV>(v, g_red_smem);
    double *buf = rc.partials + (size_t)rc.parity * NVMAX * rc.G;
    rc.parity ^= 1;
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) buf[(size_t)k * rc.G + blockIdx.x] = v[k];
    if (!grid_sync(gb, err)) return false;
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = warp_sum_partials(buf + (size_t)k * rc.G, rc.G);
            if (threadIdx.x == 0) v[k] = s;
        }
    }
    return true;
}

// scalars broadcast from thread 0 to the block
__shared__ double g_bc[8];

// One SELL row: the loads of four entries are issued before their FMAs, so a
// thread keeps several independent gathers in flight (rows hold 4-7 entries).
__device__ __forceinline__ double row_dot(const SellView &A, int i, const double *__restrict__ x) {
    int s = i >> 5;
    int e = A.sl_ptr[s] + (i & 31);
    int w = A.sl_w[s];
    double acc = 0.0;
    int k = 0;
    for (; k + 4 <= w; k += 4, e += 128) {
        int c0 = __ldg(A.col + e), c1 = __ldg(A.col + e + 32), c2 = __ldg(A.col + e + 64), c3 = __ldg(A.col + e + 96);
        double a0 = __ldg(A.val + e), a1 = __ldg(A.val + e + 32), a2 = __ldg(A.val + e + 64), a3 = __ldg(A.val + e + 96);
        double x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
        acc += a0 * x0;
        acc += a1 * x1;
        acc += a2 * x2;
        acc += a3 * x3;
    }
    for (; k < w; ++k, e += 32) acc += __ldg(A.val + e) * x[__ldg(A.col + e)];
    return acc;
}

// y_c = A (dinv .* x_c) for NR right-hand sides, skipping inactive ones.
template <int NR>
__device__ __forceinline__ void row_dot_scaled(const SellView &A, int i, const double *__restrict__ dinv,
                                               const double *__restrict__ x, int n, const bool (&act)[3],
                                               double (&y)[NR]) {
    int s = i >> 5;
    int e = A.sl_ptr[s] + (i & 31);
    int w = A.sl_w[s];
#pragma unroll
    for (int c = 0; c < NR; ++c) y[c] = 0.0;
    for (int k = 0; k < w; ++k, e += 32) {
        double a = A.val[e];
        int j = A.col[e];
        double d = dinv[j];
#pragma unroll
        for (int c = 0; c < NR; ++c)
            if (act[c]) y[c] += a * (d * x[(size_t)c * n + j]);
    }
}

__global__ void k_jacobi_dinv(SellView A, double omega, int jacobi, double *dinv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    if (!jacobi) {
        dinv[i] = 1.0;
        return;
    }
    double d = A.val[A.sl_ptr[i >> 5] + (i & 31)];
    dinv[i] = omega / d;
}

__global__ void k_spmv(SellView A, const double *__restrict__ x, double *__restrict__ y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    y[i] = row_dot(A, i, x);
}

__global__ void k_jacobi_apply(SellView A, double omega, const double *c, double *y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    double d = A.val[A.sl_ptr[i >> 5] + (i & 31)];
    y[i] = omega * c[i] / d;
}

__global__ void k_zero(double *x, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = 0.0;
}

struct CgArgs {
    SellView A;
    const double *b;
    double *x, *r, *p, *q;
    const double *dinv;
    double *partials;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit;
    double eps;
    unsigned long long *ts;  // optional phase timestamps (KrylovWork::phase_ts)
};

// Phase timestamps for profiling: block 0 records %globaltimer at the phase
// boundaries of the first PHASE_TS_ITERS iterations (4 per iteration).
constexpr int PHASE_TS_ITERS = 64;
__device__ __forceinline__ void stamp(unsigned long long *ts, int it, int k) {
    if (ts && blockIdx.x == 0 && threadIdx.x == 0 && it >= 1 && it <= PHASE_TS_ITERS) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        ts[(it - 1) * 4 + k] = t;
    }
}

// CG kernels run 1024-thread blocks, one per SM: 152 arrivals per grid barrier
// instead of 4x as many, and the vector phases walk 4 rows per thread with
// 16-byte loads so each thread keeps several loads in flight.
constexpr int KBC = 1024;

__device__ __forceinline__ double2 ld2(const double *p, int j) { return reinterpret_cast<const double2 *>(p)[j]; }
__device__ __forceinline__ void st2(double *p, int j, double2 v) { reinterpret_cast<double2 *>(p)[j] = v; }
__device__ __forceinline__ float4 ld4(const float *p, int j) { return reinterpret_cast<const float4 *>(p)[j]; }
__device__ __forceinline__ void st4(float *p, int j, float4 v) { reinterpret_cast<float4 *>(p)[j] = v; }

__global__ void __launch_bounds__(KBC, 1) k_cg(CgArgs a) {
    const int n = a.A.n;
    const int T = gridDim.x * KBC;
    const int t0 = blockIdx.x * KBC + threadIdx.x;
    const int n4 = n >> 2;  // rows 4*n4 .. n-1 form the scalar tail
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const double *__restrict__ dinv = a.dinv;

    // r = b - A x; ||b||^2, ||r||^2, rho = r . M^-1 r
    double v3[3] = {0.0, 0.0, 0.0};
    for (int i = t0; i < n; i += T) {
        double bi = a.b[i];
        double ri = bi - row_dot(a.A, i, a.x);
        a.r[i] = ri;
        v3[0] += bi * bi;
        v3[1] += ri * ri;
        v3[2] += ri * (dinv[i] * ri);
    }
    if (!grid_reduce_t0<3>(v3, rc, a.gb, err)) return;
    // scalar state lives in thread 0; the block reads the broadcast copies
    double bnorm = 1.0, res = 0.0, rho = 0.0;
    if (threadIdx.x == 0) {
        bnorm = sqrt(v3[0]);
        if (bnorm == 0.0) bnorm = 1.0;
        res = sqrt(v3[1]) / bnorm;
        rho = v3[2];
        g_bc[0] = res;
        g_bc[1] = 0.0;  // beta
    }
    __syncthreads();
    int it = 0, status = DEV_OK;
    for (;;) {
        double resb = g_bc[0], beta = g_bc[1];
        __syncthreads();
        if (resb < a.eps || it >= a.maxit) break;
        if (!isfinite(resb)) { status = DEV_NONFINITE; break; }
        ++it;
        stamp(a.ts, it, 0);
        // p = M^-1 r + beta p  (beta = 0 and p read as 0 on the first iteration)
        for (int j = t0; j < n4; j += T) {
            double2 r0 = ld2(a.r, 2 * j), r1 = ld2(a.r, 2 * j + 1);
            double2 d0 = ld2(dinv, 2 * j), d1 = ld2(dinv, 2 * j + 1);
            double2 p0 = make_double2(0.0, 0.0), p1 = p0;
            if (it > 1) { p0 = ld2(a.p, 2 * j); p1 = ld2(a.p, 2 * j + 1); }
            p0.x = d0.x * r0.x + beta * p0.x;
            p0.y = d0.y * r0.y + beta * p0.y;
            p1.x = d1.x * r1.x + beta * p1.x;
            p1.y = d1.y * r1.y + beta * p1.y;
            st2(a.p, 2 * j, p0);
            st2(a.p, 2 * j + 1, p1);
        }
        for (int i = 4 * n4 + t0; i < n; i += T) {
            double z = dinv[i] * a.r[i];
            a.p[i] = (it == 1) ? z : z + beta * a.p[i];
        }
        if (!grid_sync(a.gb, err)) return;
        stamp(a.ts, it, 1);
        double v1[1] = {0.0};
        for (int i = t0; i < n; i += T) {
            double qi = row_dot(a.A, i, a.p);
            a.q[i] = qi;
            v1[0] += a.p[i] * qi;
        }
        if (!grid_reduce_t0<1>(v1, rc, a.gb, err)) return;
        stamp(a.ts, it, 2);
        if (threadIdx.x == 0) {
            g_bc[2] = v1[0] == 0.0 ? 0.0 : rho / v1[0];
            g_bc[3] = v1[0] == 0.0 ? 1.0 : 0.0;
        }
        __syncthreads();
        double alpha = g_bc[2];
        if (g_bc[3] != 0.0) { status = DEV_BREAKDOWN; break; }
        double v2[2] = {0.0, 0.0};
        for (int j = t0; j < n4; j += T) {
            double2 p0 = ld2(a.p, 2 * j), p1 = ld2(a.p, 2 * j + 1);
            double2 q0 = ld2(a.q, 2 * j), q1 = ld2(a.q, 2 * j + 1);
            double2 x0 = ld2(a.x, 2 * j), x1 = ld2(a.x, 2 * j + 1);
            double2 r0 = ld2(a.r, 2 * j), r1 = ld2(a.r, 2 * j + 1);
            double2 d0 = ld2(dinv, 2 * j), d1 = ld2(dinv, 2 * j + 1);
            x0.x += alpha * p0.x; x0.y += alpha * p0.y; x1.x += alpha * p1.x; x1.y += alpha * p1.y;
            r0.x -= alpha * q0.x; r0.y -= alpha * q0.y; r1.x -= alpha * q1.x; r1.y -= alpha * q1.y;
            st2(a.x, 2 * j, x0);
            st2(a.x, 2 * j + 1, x1);
            st2(a.r, 2 * j, r0);
            st2(a.r, 2 * j + 1, r1);
            v2[0] += r0.x * r0.x; v2[1] += r0.x * (d0.x * r0.x);
            v2[0] += r0.y * r0.y; v2[1] += r0.y * (d0.y * r0.y);
            v2[0] += r1.x * r1.x; v2[1] += r1.x * (d1.x * r1.x);
            v2[0] += r1.y * r1.y; v2[1] += r1.y * (d1.y * r1.y);
        }
        for (int i = 4 * n4 + t0; i < n; i += T) {
            double pi = a.p[i], qi = a.q[i];
            a.x[i] += alpha * pi;
            double ri = a.r[i] - alpha * qi;
            a.r[i] = ri;
            v2[0] += ri * ri;
            v2[1] += ri * (dinv[i] * ri);
        }
        if (!grid_reduce_t0<2>(v2, rc, a.gb, err)) return;
        stamp(a.ts, it, 3);
        if (threadIdx.x == 0) {
            res = sqrt(v2[0]) / bnorm;
            g_bc[0] = res;
            g_bc[1] = v2[1] / rho;
            rho = v2[1];
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (status == DEV_OK && !(res < a.eps)) status = isfinite(res) ? DEV_MAXITER : DEV_NONFINITE;
        a.info->status[0] = status;
        a.info->iters[0] = it;
        a.info->res[0] = res;
    }
}

// ---------------------------------------------------------------------------
// Mixed precision: Jacobi-CG whose recurrences (p, q, r and the correction e)
// run in FP32, with reliable updates (Sleijpen & van der Vorst, "Reliable
// updated residuals in hybrid Bi-CG methods", Computing 56, 1996): when the
// FP32 residual has fallen by inner_tol since the last update, e is added to
// the FP64 solution, e is zeroed, the FP64 residual b - A x replaces the FP32
// one and the search direction is kept, so the Krylov process is not
// restarted.  Convergence is decided on that FP64 residual only.
__device__ __forceinline__ float row_dot32(const SellView &A, const float *__restrict__ val32, int i,
                                           const float *__restrict__ x) {
    int s = i >> 5;
    int e = A.sl_ptr[s] + (i & 31);
    int w = A.sl_w[s];
    float acc = 0.f;
    int k = 0;
    for (; k + 4 <= w; k += 4, e += 128) {
        int c0 = __ldg(A.col + e), c1 = __ldg(A.col + e + 32), c2 = __ldg(A.col + e + 64), c3 = __ldg(A.col + e + 96);
        float a0 = __ldg(val32 + e), a1 = __ldg(val32 + e + 32), a2 = __ldg(val32 + e + 64), a3 = __ldg(val32 + e + 96);
        float x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
        acc = fmaf(a0, x0, acc);
        acc = fmaf(a1, x1, acc);
        acc = fmaf(a2, x2, acc);
        acc = fmaf(a3, x3, acc);
    }
    for (; k < w; ++k, e += 32) acc = fmaf(__ldg(val32 + e), x[__ldg(A.col + e)], acc);
    return acc;
}

struct CgMixedArgs {
    SellView A;  // FP64 values
    const float *val32;
    const double *b;
    double *x, *r64;
    float *r32, *p32, *q32, *e32;
    const float *dinv32;
    double *partials;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit;
    double eps, inner_tol;
    unsigned long long *ts;
};

__global__ void __launch_bounds__(KBC, 1) k_cg_mixed(CgMixedArgs a) {
    const int n = a.A.n;
    const int T = gridDim.x * KBC;
    const int t0 = blockIdx.x * KBC + threadIdx.x;
    const int n4 = n >> 2;  // float4 chunks; rows 4*n4 .. n-1 form the scalar tail
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const float *__restrict__ dinv = a.dinv32;

    // FP64 residual of the initial guess and its FP32 copy.  Per-thread partial
    // sums of FP32 products run over a few rows in FP32; FP64 across threads.
    double v3[3] = {0.0, 0.0, 0.0};
    float f2 = 0.f;
    for (int i = t0; i < n; i += T) {
        double bi = a.b[i];
        double ri = bi - row_dot(a.A, i, a.x);
        float rf = (float)ri;
        a.r32[i] = rf;
        a.e32[i] = 0.f;
        v3[0] += bi * bi;
        v3[1] += ri * ri;
        f2 = fmaf(rf, dinv[i] * rf, f2);
    }
    v3[2] = (double)f2;
    if (!grid_reduce_t0<3>(v3, rc, a.gb, err)) return;
    // thread-0 scalar state
    double bnorm = 1.0, bb = 0.0, res = 0.0, rho = 0.0, rr_ref = 0.0;
    const double d2 = a.inner_tol * a.inner_tol, e2 = a.eps * a.eps;
    if (threadIdx.x == 0) {
        bb = v3[0];
        bnorm = sqrt(bb);
        if (bnorm == 0.0) { bnorm = 1.0; bb = 1.0; }
        res = sqrt(v3[1]) / bnorm;
        rr_ref = v3[1];
        rho = v3[2];
        g_bc[0] = res;
        g_bc[1] = 0.0;
    }
    __syncthreads();
    int total = 0, nupd = 0, status = DEV_OK;
    for (;;) {
        double resb = g_bc[0];
        float beta = (float)g_bc[1];
        __syncthreads();
        if (resb < a.eps || total >= a.maxit) break;  // resb: FP64 residual of the last update
        if (!isfinite(resb)) { status = DEV_NONFINITE; break; }
        ++total;
        stamp(a.ts, total, 0);
        for (int j = t0; j < n4; j += T) {
            float4 r = ld4(a.r32, j), d = ld4(dinv, j);
            float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
            if (total > 1) p = ld4(a.p32, j);
            p.x = fmaf(beta, p.x, d.x * r.x);
            p.y = fmaf(beta, p.y, d.y * r.y);
            p.z = fmaf(beta, p.z, d.z * r.z);
            p.w = fmaf(beta, p.w, d.w * r.w);
            st4(a.p32, j, p);
        }
        for (int i = 4 * n4 + t0; i < n; i += T) {
            float z = dinv[i] * a.r32[i];
            a.p32[i] = (total == 1) ? z : fmaf(beta, a.p32[i], z);
        }
        if (!grid_sync(a.gb, err)) return;
        stamp(a.ts, total, 1);
        float g0 = 0.f;
        for (int i = t0; i < n; i += T) {
            float qi = row_dot32(a.A, a.val32, i, a.p32);
            a.q32[i] = qi;
            g0 = fmaf(a.p32[i], qi, g0);
        }
        double v1[1] = {(double)g0};
        if (!grid_reduce_t0<1>(v1, rc, a.gb, err)) return;
        stamp(a.ts, total, 2);
        if (threadIdx.x == 0) {
            g_bc[2] = v1[0] == 0.0 ? 0.0 : rho / v1[0];
            g_bc[3] = v1[0] == 0.0 ? 1.0 : 0.0;
        }
        __syncthreads();
        float alpha = (float)g_bc[2];
        if (g_bc[3] != 0.0) { status = DEV_BREAKDOWN; break; }
        float h0 = 0.f, h1 = 0.f;
        for (int j = t0; j < n4; j += T) {
            float4 p = ld4(a.p32, j), q = ld4(a.q32, j), e = ld4(a.e32, j), r = ld4(a.r32, j), d = ld4(dinv, j);
            e.x = fmaf(alpha, p.x, e.x); e.y = fmaf(alpha, p.y, e.y);
            e.z = fmaf(alpha, p.z, e.z); e.w = fmaf(alpha, p.w, e.w);
            r.x = fmaf(-alpha, q.x, r.x); r.y = fmaf(-alpha, q.y, r.y);
            r.z = fmaf(-alpha, q.z, r.z); r.w = fmaf(-alpha, q.w, r.w);
            st4(a.e32, j, e);
            st4(a.r32, j, r);
            h0 = fmaf(r.x, r.x, h0); h1 = fmaf(r.x, d.x * r.x, h1);
            h0 = fmaf(r.y, r.y, h0); h1 = fmaf(r.y, d.y * r.y, h1);
            h0 = fmaf(r.z, r.z, h0); h1 = fmaf(r.z, d.z * r.z, h1);
            h0 = fmaf(r.w, r.w, h0); h1 = fmaf(r.w, d.w * r.w, h1);
        }
        for (int i = 4 * n4 + t0; i < n; i += T) {
            a.e32[i] = fmaf(alpha, a.p32[i], a.e32[i]);
            float ri = fmaf(-alpha, a.q32[i], a.r32[i]);
            a.r32[i] = ri;
            h0 = fmaf(ri, ri, h0);
            h1 = fmaf(ri, dinv[i] * ri, h1);
        }
        double w2[2] = {(double)h0, (double)h1};
        if (!grid_reduce_t0<2>(w2, rc, a.gb, err)) return;
        stamp(a.ts, total, 3);
        if (threadIdx.x == 0) {
            // reliable update once the FP32 residual fell by inner_tol since the
            // last one, when it looks converged, or at the iteration cap
            bool upd = w2[0] <= d2 * rr_ref || w2[0] <= e2 * bb || total >= a.maxit || !(w2[0] == w2[0]);
            if (!upd) {
                g_bc[1] = w2[1] / rho;
                rho = w2[1];
            }
            g_bc[4] = upd ? 1.0 : 0.0;
        }
        __syncthreads();
        if (g_bc[4] != 0.0) {
            for (int j = t0; j < n4; j += T) {
                float4 e = ld4(a.e32, j);
                double2 x0 = ld2(a.x, 2 * j), x1 = ld2(a.x, 2 * j + 1);
                x0.x += (double)e.x; x0.y += (double)e.y; x1.x += (double)e.z; x1.y += (double)e.w;
                st2(a.x, 2 * j, x0);
                st2(a.x, 2 * j + 1, x1);
                st4(a.e32, j, make_float4(0.f, 0.f, 0.f, 0.f));
            }
            for (int i = 4 * n4 + t0; i < n; i += T) {
                a.x[i] += (double)a.e32[i];
                a.e32[i] = 0.f;
            }
            if (!grid_sync(a.gb, err)) return;
            double u[2] = {0.0, 0.0};
            float fz = 0.f;
            for (int i = t0; i < n; i += T) {
                double ri = a.b[i] - row_dot(a.A, i, a.x);
                float rf = (float)ri;
                a.r32[i] = rf;
                u[0] += ri * ri;
                fz = fmaf(rf, dinv[i] * rf, fz);
            }
            u[1] = (double)fz;
            if (!grid_reduce_t0<2>(u, rc, a.gb, err)) return;
            if (threadIdx.x == 0) {
                res = sqrt(u[0]) / bnorm;
                rr_ref = u[0];
                g_bc[0] = res;
                g_bc[1] = u[1] / rho;  // keep the direction: beta from the replaced residual
                rho = u[1];
                ++nupd;
            }
            __syncthreads();
        }
    }
    if (status == DEV_BREAKDOWN)  // keep the correction gathered so far
        for (int i = t0; i < n; i += T) a.x[i] += (double)a.e32[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (status == DEV_OK && !(res < a.eps)) status = isfinite(res) ? DEV_MAXITER : DEV_NONFINITE;
        a.info->status[0] = status;
        a.info->iters[0] = total;
        a.info->res[0] = res;
        a.info->refinements = nupd;
    }
}

__global__ void k_to_fp32(long n, const double *src, float *dst) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

__global__ void k_dinv32(SellView A, double omega, float *dinv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    dinv[i] = (float)(omega / A.val[A.sl_ptr[i >> 5] + (i & 31)]);
}

struct BicgArgs {
    SellView A;
    const double *b[3];
    double *x[3];
    double *r, *rt, *p, *v, *s, *t;
    const double *dinv;
    double *partials;
    GridBarrier *gb;
    SolveInfo *info;
    int maxit;
    double eps;
};

template <int NR>
__global__ void __launch_bounds__(KB) k_bicgstab(BicgArgs a) {
    const int n = a.A.n;
    const int T = gridDim.x * KB;
    const int t0 = blockIdx.x * KB + threadIdx.x;
    int *err = &a.info->err;
    RedCtx rc{a.partials, (int)gridDim.x, 0};
    const double *__restrict__ dinv = a.dinv;
    const size_t N = (size_t)n;

    double bnorm[NR], res[NR], rho[NR], rho_prev[NR], alpha[NR], omg[NR], beta[NR], snorm[NR];
    int it[NR], status[NR];
    bool done[NR], act[3] = {false, false, false}, early[3] = {false, false, false};
    {
        double v[2 * NR];
#pragma unroll
        for (int c = 0; c < 2 * NR; ++c) v[c] = 0.0;
        for (int i = t0; i < n; i += T) {
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                double bi = a.b[c][i];
                double ri = bi - row_dot(a.A, i, a.x[c]);
                a.r[c * N + i] = ri;
                a.rt[c * N + i] = ri;
                v[c] += bi * bi;
                v[NR + c] += ri * ri;
            }
        }
        if (!grid_reduce<2 * NR>(v, rc, a.gb, err)) return;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            bnorm[c] = sqrt(v[c]);
            if (bnorm[c] == 0.0) bnorm[c] = 1.0;
            res[c] = sqrt(v[NR + c]) / bnorm[c];
            rho[c] = v[NR + c];
            rho_prev[c] = alpha[c] = omg[c] = 1.0;
            it[c] = 0;
            status[c] = DEV_OK;
            done[c] = false;
        }
    }
    for (;;) {
        bool any = false;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            act[c] = !done[c] && !(res[c] < a.eps) && it[c] < a.maxit;
            if (act[c] && !isfinite(res[c])) { done[c] = true; status[c] = DEV_NONFINITE; act[c] = false; }
            if (act[c] && rho[c] == 0.0) { done[c] = true; status[c] = DEV_BREAKDOWN; act[c] = false; }
            if (act[c]) {
                ++it[c];
                any = true;
                beta[c] = (it[c] == 1) ? 0.0 : (rho[c] / rho_prev[c]) * (alpha[c] / omg[c]);
            }
        }
        if (!any) break;
        // p = r + beta (p - omega v)
        for (int i = t0; i < n; i += T) {
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                if (!act[c]) continue;
                size_t k = c * N + i;
                a.p[k] = (it[c] == 1) ? a.r[k] : a.r[k] + beta[c] * (a.p[k] - omg[c] * a.v[k]);
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
                row_dot_scaled<NR>(a.A, i, dinv, a.p, n, act, y);
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act[c]) continue;
                    a.v[c * N + i] = y[c];
                    red[c] += a.rt[c * N + i] * y[c];
                }
            }
            if (!grid_reduce<NR>(red, rc, a.gb, err)) return;
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                if (!act[c]) continue;
                if (red[c] == 0.0) { done[c] = true; status[c] = DEV_BREAKDOWN; act[c] = false; continue; }
                alpha[c] = rho[c] / red[c];
            }
        }
        // s = r - alpha v ; ||s||
        {
            double red[NR];
#pragma unroll
            for (int c = 0; c < NR; ++c) red[c] = 0.0;
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
            if (!grid_reduce<NR>(red, rc, a.gb, err)) return;
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                early[c] = false;
                if (!act[c]) continue;
                snorm[c] = sqrt(red[c]) / bnorm[c];
                early[c] = snorm[c] < a.eps;
            }
        }
        // t = A M^-1 s ; t.s, t.t
        {
            bool act2[3] = {false, false, false};
#pragma unroll
            for (int c = 0; c < NR; ++c) act2[c] = act[c] && !early[c];
            double red[2 * NR];
#pragma unroll
            for (int c = 0; c < 2 * NR; ++c) red[c] = 0.0;
            for (int i = t0; i < n; i += T) {
                double y[NR];
                row_dot_scaled<NR>(a.A, i, dinv, a.s, n, act2, y);
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act2[c]) continue;
                    size_t k = c * N + i;
                    a.t[k] = y[c];
                    red[c] += y[c] * a.s[k];
                    red[NR + c] += y[c] * y[c];
                }
            }
            if (!grid_reduce<2 * NR>(red, rc, a.gb, err)) return;
#pragma unroll
            for (int c = 0; c < NR; ++c)
                if (act2[c]) omg[c] = red[NR + c] != 0.0 ? red[c] / red[NR + c] : 0.0;
        }
        // x += alpha M^-1 p + omega M^-1 s ; r = s - omega t
        {
            double red[2 * NR];
#pragma unroll
            for (int c = 0; c < 2 * NR; ++c) red[c] = 0.0;
            for (int i = t0; i < n; i += T) {
                double di = dinv[i];
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    if (!act[c]) continue;
                    size_t k = c * N + i;
                    double ph = di * a.p[k];
                    if (early[c]) {
                        a.x[c][i] += alpha[c] * ph;
                    } else {
                        double sh = di * a.s[k];
                        a.x[c][i] += alpha[c] * ph + omg[c] * sh;
                        double ri = a.s[k] - omg[c] * a.t[k];
                        a.r[k] = ri;
                        red[c] += ri * ri;
                        red[NR + c] += a.rt[k] * ri;
                    }
                }
            }
            if (!grid_reduce<2 * NR>(red, rc, a.gb, err)) return;
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                if (!act[c]) continue;
                if (early[c]) {
                    res[c] = snorm[c];
                    done[c] = true;
                } else {
                    res[c] = sqrt(red[c]) / bnorm[c];
                    rho_prev[c] = rho[c];
                    rho[c] = red[NR + c];
                    if (omg[c] == 0.0 && !(res[c] < a.eps)) { done[c] = true; status[c] = DEV_BREAKDOWN; }
                }
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            int st = status[c];
            if (st == DEV_OK && !(res[c] < a.eps)) st = isfinite(res[c]) ? DEV_MAXITER : DEV_NONFINITE;
            a.info->status[c] = st;
            a.info->iters[c] = it[c];
            a.info->res[c] = res[c];
        }
    }
}

int g_num_sms = 0;

int num_sms() {
    if (!g_num_sms) {
        int dev;
        SYSU_CUDA(cudaGetDevice(&dev));
        SYSU_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
        int coop = 0;
        SYSU_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) throw CaseError{"device does not support cooperative launch"};
    }
    return g_num_sms;
}

template <class K>
int coresident_blocks(K kernel, int block = KB) {
    int per_sm = 0;
    SYSU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0));
    if (per_sm < 1) throw CaseError{"persistent Krylov kernel cannot be resident"};
    return per_sm * num_sms();
}

SellView view(const SellDev &A, const double *val) {
    return SellView{A.n, A.nslices, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val};
}

int grid_for(int n, int max_blocks, int block = KB) {
    int want = (n + block - 1) / block;
    return std::max(1, std::min(want, max_blocks));
}

// the vector phases of the CG kernels use 16-byte loads
void check_aligned16(std::initializer_list<const void *> ptrs) {
    for (const void *p : ptrs)
        if (reinterpret_cast<uintptr_t>(p) % 16 != 0) throw CaseError{"CG vectors must be 16-byte aligned"};
}

}  // namespace

void KrylovWork::ensure(int n_, int nrhs_, int max_blocks_, cudaStream_t st) {
    if (n_ <= n && nrhs_ <= nrhs && max_blocks_ <= max_blocks) return;
    n = std::max(n, n_);
    nrhs = std::max(nrhs, nrhs_);
    max_blocks = std::max(max_blocks, max_blocks_);
    size_t m = (size_t)n * nrhs;
    r.alloc(m); rt.alloc(m); p.alloc(m); v.alloc(m); s.alloc(m); t.alloc(m);
    dinv.alloc(n);
    partials.alloc((size_t)2 * NVMAX * max_blocks);
    barrier.alloc(1);
    barrier.zero(st);
}

void KrylovWork::ensure32(int n_, cudaStream_t st) {
    if (r32.size() >= (size_t)n_) return;
    r32.alloc(n_); p32.alloc(n_); q32.alloc(n_); e32.alloc(n_); dinv32.alloc(n_);
    (void)st;
}

void sell_to_fp32(const SellDev &A, const double *val, float *val32, cudaStream_t st) {
    if (A.nnz == 0) return;
    { k_to_fp32<<<(unsigned)((A.nnz + KB - 1) / KB), KB, 0, st>>>(A.nnz, val, val32); ++::sysu::g_launches; }
    SYSU_CUDA(cudaGetLastError());
}

void cg_solve_mixed(const SellDev &A, const double *val, const float *val32, const double *b, double *x,
                    bool x0_zero, const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = coresident_blocks(k_cg_mixed, KBC);
    w.ensure(n, 1, maxb, st);
    w.ensure32(n, st);
    check_aligned16({x, w.r32.get(), w.p32.get(), w.q32.get(), w.e32.get(), w.dinv32.get()});
    SellView V = view(A, val);
    { k_dinv32<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, w.dinv32.get()); ++::sysu::g_launches; }
    if (x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    CgMixedArgs a{};
    a.A = V;
    a.val32 = val32;
    a.b = b;
    a.x = x;
    a.r64 = w.r.get();
    a.r32 = w.r32.get(); a.p32 = w.p32.get(); a.q32 = w.q32.get(); a.e32 = w.e32.get();
    a.dinv32 = w.dinv32.get();
    a.partials = w.partials.get();
    a.gb = w.barrier.get();
    a.info = info;
    a.maxit = o.maxit;
    a.eps = o.eps;
    a.inner_tol = o.inner_tol;
    a.ts = w.phase_ts;
    void *args[] = {&a};
    int G = grid_for(n, maxb, KBC);
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_cg_mixed, dim3(G), dim3(KBC), args, 0, st)); ++::sysu::g_launches; }
}

void spmv(const SellDev &A, const double *val, const double *x, double *y, cudaStream_t st) {
    if (A.n == 0) return;
    { k_spmv<<<(A.n + KB - 1) / KB, KB, 0, st>>>(view(A, val), x, y); ++::sysu::g_launches; }
    SYSU_CUDA(cudaGetLastError());
}

void jacobi_apply(const SellDev &A, const double *val, double omega, const double *c, double *y, cudaStream_t st) {
    if (A.n == 0) return;
    { k_jacobi_apply<<<(A.n + KB - 1) / KB, KB, 0, st>>>(view(A, val), omega, c, y); ++::sysu::g_launches; }
    SYSU_CUDA(cudaGetLastError());
}

void cg_solve(const SellDev &A, const double *val, const double *b, double *x, bool x0_zero,
              const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    static int maxb = 0;
    if (!maxb) maxb = coresident_blocks(k_cg, KBC);
    w.ensure(n, 1, maxb, st);
    check_aligned16({x, w.r.get(), w.p.get(), w.v.get(), w.dinv.get()});
    SellView V = view(A, val);
    { k_jacobi_dinv<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, o.jacobi ? 1 : 0, w.dinv.get()); ++::sysu::g_launches; }
    if (x0_zero) { k_zero<<<(n + KB - 1) / KB, KB, 0, st>>>(x, n); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    CgArgs a{V, b, x, w.r.get(), w.p.get(), w.v.get(), w.dinv.get(), w.partials.get(), w.barrier.get(), info,
             o.maxit, o.eps, w.phase_ts};
    void *args[] = {&a};
    int G = grid_for(n, maxb, KBC);
    { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_cg, dim3(G), dim3(KBC), args, 0, st)); ++::sysu::g_launches; }
}

void bicgstab_solve(const SellDev &A, const double *val, int nrhs, const double *const *b, double *const *x,
                    const KrylovOpts &o, KrylovWork &w, SolveInfo *info, cudaStream_t st) {
    int n = A.n;
    if (n == 0) return;
    if (nrhs < 1 || nrhs > 3) throw CaseError{"bicgstab_solve: 1..3 right-hand sides"};
    static int maxb1 = 0, maxb3 = 0;
    if (!maxb1) {
        maxb1 = coresident_blocks(k_bicgstab<1>);
        maxb3 = coresident_blocks(k_bicgstab<3>);
    }
    int maxb = (nrhs == 1) ? maxb1 : maxb3;
    w.ensure(n, nrhs == 1 ? 1 : 3, std::max(maxb1, maxb3), st);
    SellView V = view(A, val);
    { k_jacobi_dinv<<<(n + KB - 1) / KB, KB, 0, st>>>(V, o.omega, o.jacobi ? 1 : 0, w.dinv.get()); ++::sysu::g_launches; }
    SYSU_CUDA(cudaMemsetAsync(info, 0, sizeof(SolveInfo), st));
    BicgArgs a{};
    a.A = V;
    for (int c = 0; c < 3; ++c) {
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
    int G = grid_for(n, maxb);
    if (nrhs == 1)
        { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_bicgstab<1>, dim3(G), dim3(KB), args, 0, st)); ++::sysu::g_launches; }
    else if (nrhs == 2)
        throw CaseError{"bicgstab_solve: use 1 or 3 right-hand sides"};
    else
        { SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_bicgstab<3>, dim3(G), dim3(KB), args, 0, st)); ++::sysu::g_launches; }
}

}  // namespace sysu
