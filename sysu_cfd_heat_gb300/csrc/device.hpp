// Device-side building blocks shared by the finite-volume and Krylov kernels:
// error checking, owning device buffers, deterministic reductions and a
// grid-wide barrier whose every wait is bounded.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "case.hpp"

namespace sysu {

#define SYSU_CUDA(call)                                                                      \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            throw ::sysu::CaseError{std::string(#call) + ": " + cudaGetErrorString(e_)};    \
    } while (0)

// Number of kernels this library has launched (all solvers, all threads).
extern std::atomic<long> g_launches;

// Owning device allocation.
template <class T>
class DevBuf {
  public:
    DevBuf() = default;
    explicit DevBuf(size_t n) { alloc(n); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { release(); p_ = o.p_; n_ = o.n_; o.p_ = nullptr; o.n_ = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t n) {
        release();
        n_ = n;
        if (n) SYSU_CUDA(cudaMalloc((void **)&p_, n * sizeof(T)));
    }
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    void upload(const T *h, size_t n, cudaStream_t s) {
        if (n > n_) throw CaseError{"upload larger than buffer"};
        if (n) SYSU_CUDA(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T> &h, cudaStream_t s) {
        if (h.size() != n_) alloc(h.size());
        upload(h.data(), h.size(), s);
    }
    void download(T *h, size_t n, cudaStream_t s) const {
        if (n > n_) throw CaseError{"download larger than buffer"};
        if (n) SYSU_CUDA(cudaMemcpyAsync(h, p_, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void zero(cudaStream_t s) {
        if (n_) SYSU_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), s));
    }
    T *get() const { return p_; }
    size_t size() const { return n_; }

  private:
    T *p_ = nullptr;
    size_t n_ = 0;
};

// Grid barrier state for persistent (cooperatively launched) kernels.
struct GridBarrier {
    unsigned int count;
    unsigned int gen;
};

// Status words written by device code instead of trapping.
enum DevStatus : int {
    DEV_OK = 0,
    DEV_MAXITER = 1,
    DEV_BREAKDOWN = 2,
    DEV_BARRIER_TIMEOUT = 3,
    DEV_NONFINITE = 4,
    // mixed-precision solves: three FP64 updates in a row did not halve the
    // residual norm (FP32's rounding floor); the FP64 solve launched behind it
    // finishes from the current x and reports its own status
    DEV_STALLED = 5,
};

#ifdef __CUDACC__

constexpr unsigned FULL_MASK = 0xffffffffu;
// A few seconds of polling (each poll is an L2 round trip); a wait that is
// still not over by then records DEV_BARRIER_TIMEOUT and gives up.
constexpr long long BARRIER_SPIN_LIMIT = 4000000LL;

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier of a cooperative launch on one 32-bit counter whose low 31 bits
// are zero between barriers: block 0 adds 2^31 - (blocks - 1), every other
// block adds 1, so the counter's top bit flips exactly when the last block
// arrives and returns the low bits to zero.  One release atomic per block to
// arrive, acquire loads to wait (no reset step, no separate generation word).
// Every block calls it the same number of times; the counter must be zero (or
// 2^31) when the launch starts -- the solvers clear it before each launch.
// Returns false (and sets *err) if the wait timed out, in which case the caller
// must leave the kernel.
__device__ __forceinline__ bool grid_sync(GridBarrier *gb, int *err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
        unsigned old;
        asm volatile("atom.add.release.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(&gb->count), "r"(inc) : "memory");
        long long spins = 0;
        while (((ld_acquire(&gb->count) ^ old) & 0x80000000u) == 0u) {
            if (++spins > BARRIER_SPIN_LIMIT) {
                atomicExch(err, (int)DEV_BARRIER_TIMEOUT);
                ok = 0;
                break;
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Deterministic block sum of NV values per thread; result valid in every thread.
// smem must hold NV * (blockDim.x/32) doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem) {
#pragma unroll
    for (int k = 0; k < NV; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(FULL_MASK, v[k], o);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) smem[k * nw + warp] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += smem[k * nw + w];
        v[k] = s;
    }
}

// Deterministic block sum of NV values per thread; the result is valid in
// thread 0 only (warp 0 alone combines the warp sums, which keeps the FP64
// work per block small).  smem must hold NV * (blockDim.x/32) doubles.
template <int NV>
__device__ __forceinline__ void block_sum_t0(double (&v)[NV], double *smem) {
#pragma unroll
    for (int k = 0; k < NV; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(FULL_MASK, v[k], o);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) smem[k * nw + warp] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += smem[k * nw + w];
            v[k] = s;
        }
    }
}

// Sum of `count` partials laid out partials[k*stride + b], b < count, computed
// by one warp in a fixed order (identical in every block); all lanes get it.
__device__ __forceinline__ double warp_sum_partials(const double *partials, int count) {
    int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int b = lane; b < count; b += 32) s += __ldcg(partials + b);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
    return s;
}

#endif  // __CUDACC__

}  // namespace sysu
