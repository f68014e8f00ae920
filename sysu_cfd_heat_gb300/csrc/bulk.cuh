// Bulk asynchronous copies (the TMA engine's 1-D form) from global memory into
// shared memory, completed on mbarriers, and a ring of copy slots that the
// persistent Krylov kernels stream their tiles through.
//
// PTX used (sm_90 and later, so sm_103a): mbarrier.init / arrive.expect_tx /
// try_wait.parity, cp.async.bulk.shared::cluster.global.mbarrier::complete_tx
// with an L2 cache-policy operand, createpolicy, fence.proxy.async.  A kernel
// that is not launched as a cluster is a one-CTA cluster, so a CTA-local shared
// address is a valid shared::cluster address.
//
// Rules the callers keep (checked on the host where they can be):
//   - global source and shared destination 16-byte aligned, sizes multiples of
//     16 bytes and > 0;
//   - every wait is bounded (COPY_WAIT_NS); on a timeout the caller records an
//     error, stops issuing, drains what it issued and leaves the kernel;
//   - a CTA never exits with a copy in flight (drain()).
#pragma once

#include <cstdint>

#include "device.hpp"

namespace sysu {

#ifdef __CUDACC__

// One second: far above any legitimate copy latency.
constexpr unsigned long long COPY_WAIT_NS = 1000000000ULL;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_timer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Make initialised mbarriers visible to the async proxy before first use.
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Non-blocking probe: has the phase with the given parity completed?
// (try_wait may suspend the thread for a system-dependent time when the phase
// is still open; test_wait returns at once.)
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait with a suspend-time hint: the warp sleeps in hardware until the
// phase completes or about `ns` nanoseconds pass, instead of spinning on issue
// slots that the producer warp of the same SM needs.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, unsigned parity, unsigned ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}

// Wait for the phase with the given parity to complete; false after
// COPY_WAIT_NS without completion.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    if (mbar_try_wait_sleep(bar, parity, 100000u)) return true;
    unsigned long long t0 = global_timer_ns();
    for (;;) {
        if (mbar_try_wait_sleep(bar, parity, 100000u)) return true;
        if (global_timer_ns() - t0 > COPY_WAIT_NS) return false;
    }
}

// L2 policies for the copies: the matrix streams through once per product and
// should not push the Krylov vectors out of L2.
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
        : "memory");
}

// Order this thread's earlier generic-proxy global writes before later
// async-proxy (bulk copy) reads of the same addresses.
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Capacity of the copy rings of the persistent kernels (slots per CTA).
struct CopyRing {
    static constexpr int DMAX = 6;
    uint64_t bar[DMAX];
};

#endif  // __CUDACC__

}  // namespace sysu
