// Device and host helpers shared by the Krylov translation units (included
// once per .cu file; everything sits in an anonymous namespace).
#pragma once

#include <algorithm>
#include <cstdint>
#include <initializer_list>

#include "exact_sum.cuh"
#include "krylov.hpp"

namespace sysu {
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

// Exact deterministic grid sums of NV <= XS_NVMAX values per thread
// (exact_sum.cuh); the sums are valid in thread 0 only.  Per-block partials are
// (exponent, 128-bit sum, nonfinite flag) in four 64-bit words, double
// buffered like grid_reduce's; rc.partials must hold 2 * XS_NVMAX * G * 4 words.
constexpr int XS_NVMAX = 3;
__shared__ long long g_xs_smem[XS_NVMAX * 32 * 4];

template <int NV>
__device__ __forceinline__ bool grid_sum_t0(double (&v)[NV], RedCtx &rc, GridBarrier *gb, int *err) {
    static_assert(NV <= XS_NVMAX, "grid_sum_t0: too many values");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        int E, nf;
        I128 S;
        xs_warp(v[k], E, S, nf);
        if (lane == 0) {
            long long *q = g_xs_smem + (k * 32 + warp) * 4;
            q[0] = E;
            q[1] = (long long)S.lo;
            q[2] = S.hi;
            q[3] = nf;
        }
    }
    __syncthreads();
    long long *buf = reinterpret_cast<long long *>(rc.partials) + (size_t)rc.parity * XS_NVMAX * rc.G * 4;
    rc.parity ^= 1;
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            int e = 0, f = 0;
            I128 s{0ull, 0ll};
            if (lane < nw) {
                const long long *q = g_xs_smem + (k * 32 + lane) * 4;
                e = (int)q[0];
                s.lo = (unsigned long long)q[1];
                s.hi = q[2];
                f = (int)q[3];
            }
            int E, nf;
            I128 S;
            xs_combine(e, s, f, 0, E, S, nf);
            if (lane == 0) {
                long long *o = buf + ((size_t)k * rc.G + blockIdx.x) * 4;
                o[0] = E;
                o[1] = (long long)S.lo;
                o[2] = S.hi;
                o[3] = nf;
            }
        }
    }
    if (!grid_sync(gb, err)) return false;
    if (warp == 0) {
        // every lane loads its blocks' partials in one pass (16-byte loads), for
        // up to XS_LANE_BLOCKS * 32 blocks at a time
        constexpr int XS_LANE_BLOCKS = 5;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const longlong2 *pk = reinterpret_cast<const longlong2 *>(buf + (size_t)k * rc.G * 4);
            int E = 0, f = 0;
            I128 t{0ull, 0ll};
            for (int c0 = 0; c0 < rc.G; c0 += 32 * XS_LANE_BLOCKS) {
                longlong2 q0[XS_LANE_BLOCKS], q1[XS_LANE_BLOCKS];
#pragma unroll
                for (int j = 0; j < XS_LANE_BLOCKS; ++j) {
                    int blk = c0 + lane + 32 * j;
                    if (blk < rc.G) {
                        q0[j] = __ldcg(pk + 2 * blk);      // exponent, low word
                        q1[j] = __ldcg(pk + 2 * blk + 1);  // high word, flag
                    } else {
                        q0[j] = make_longlong2(0, 0);
                        q1[j] = make_longlong2(0, 0);
                    }
                }
                int em = 0;
#pragma unroll
                for (int j = 0; j < XS_LANE_BLOCKS; ++j)
                    if (q0[j].y != 0 || q1[j].x != 0) em = max(em, (int)q0[j].x);
                int Ec = __reduce_max_sync(FULL_MASK, em);
                if (Ec > E) {  // rescale what earlier chunks summed (rare: more than 160 blocks)
                    t = xs_sar(t, Ec - E);
                    E = Ec;
                }
#pragma unroll
                for (int j = 0; j < XS_LANE_BLOCKS; ++j) {
                    f |= (int)q1[j].y;
                    I128 sb{(unsigned long long)q0[j].y, q1[j].x};
                    if (sb.lo != 0 || sb.hi != 0) t = xs_add(t, xs_sar(sb, E - (int)q0[j].x + XS_G));
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t = xs_add(t, xs_shfl_xor(t, o));
            int nf = __reduce_or_sync(FULL_MASK, f);
            if (lane == 0) v[k] = xs_to_double(E, t, nf, XS_G);
        }
    }
    return true;
}

// scalars broadcast from thread 0 to the block
__shared__ double g_bc[8];

// A power of two s with s^2 rr in [1, 4) (1 when rr is zero or not finite).
// The FP32 inner solves of the mixed-precision forms work on s r, so residuals
// that have become tiny (or huge) in FP64 neither underflow nor overflow in
// FP32; scaling by a power of two is exact.
__device__ __forceinline__ double pow2_scale(double rr) {
    if (!(rr > 0.0) || !isfinite(rr)) return 1.0;
    const int e = ilogb(rr);
    const int h = e >= 0 ? e / 2 : -((1 - e) / 2);  // floor(e / 2)
    return ldexp(1.0, -h);
}

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

__global__ void k_zero(double *x, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = 0.0;
}

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

// Non-persistent kernels: thread 0 of every block publishes its block's NV
// totals to part[block][NV] and counts its arrival; the last block to arrive
// adds all partials up (every thread of that block loads a strided share, then
// a block reduction in a fixed order).  Returns true in exactly one thread
// (thread 0 of the last block), which then holds the totals in v.  sm: NV * 8
// doubles of shared memory (blocks of at most 256 threads).
template <int NV>
__device__ bool grid_sums_publish(double (&v)[NV], double *part, unsigned *cnt, double *sm) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) part[(size_t)blockIdx.x * NV + k] = v[k];
        __threadfence();
        unsigned prev = atomicAdd(cnt, 1u);
        s_last = prev == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double t[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) t[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < NV; ++k) t[k] += __ldcg(part + (size_t)b * NV + k);
    block_sum_t0<NV>(t, sm);
    if (threadIdx.x != 0) return false;
    *cnt = 0;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = t[k];
    return true;
}

// Grid sums of FP64 per-thread values (block sum in FP64).
template <int NV>
__device__ bool grid_sums(double (&v)[NV], double *part, unsigned *cnt) {
    __shared__ double sm[NV * 8];
    block_sum_t0<NV>(v, sm);
    return grid_sums_publish<NV>(v, part, cnt, sm);
}

// Grid sums of FP32 per-thread partials.  The warp sums stay in FP32 (a fixed
// butterfly, so lane 0's total is the same on every run); only the warp
// totals go to FP64 for the block and grid sums.  An FP64 shuffle tree in
// every thread runs on GB300's FP64 pipe (1/64 of the FP32 rate): 6 FP64
// operations per value and thread took 10-20 us of a 2M-row vector pass.
template <int NV>
__device__ bool grid_sums_f(const float (&f)[NV], double (&v)[NV], double *part, unsigned *cnt) {
    __shared__ double sm[NV * 8];
    float g[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        g[k] = f[k];
        for (int o = 16; o > 0; o >>= 1) g[k] += __shfl_xor_sync(FULL_MASK, g[k], o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sm[k * nw + warp] = (double)g[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += sm[k * nw + w];
            v[k] = s;
        }
    return grid_sums_publish<NV>(v, part, cnt, sm);
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
}  // namespace sysu
