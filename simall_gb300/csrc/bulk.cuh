// One-dimensional bulk copies (TMA, cp.async.bulk) from global into shared
// memory with mbarrier completion, and bounded waits on them.
//
// Rules kept by the callers: both addresses and the size are multiples of 16
// bytes; the bytes announced with expect_tx equal the bytes the copies of
// that phase move; a wait gives up after kBulkWaitNs and reports it, so no
// thread spins forever on a copy that cannot complete.
#pragma once

#include <cstdint>

namespace simall {

constexpr unsigned long long kBulkWaitNs = 4000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised mbarriers visible to the async proxy (the bulk copies).
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// The producer's arrival on a phase, announcing `bytes` of copies.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// A plain arrival (a consumer releasing a buffer).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return done != 0;
}

// One potentially blocking test: the thread may be suspended in hardware
// until the phase completes or a system-dependent time limit passes, so a
// waiting warp takes no issue slots from the warps that compute.
__device__ __forceinline__ bool mbar_try(uint64_t *bar, unsigned parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return done != 0;
}

// Waits for the phase of parity `parity` to complete; false after ~4 s.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    if (mbar_try(bar, parity))
        return true;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (mbar_try(bar, parity))
            return true;
        if (globaltimer_ns() - t0 > kBulkWaitNs)
            return false;
    }
}

// Global -> shared bulk copy of `bytes` (multiple of 16, both addresses
// 16-byte aligned), completing on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// An L2 policy that evicts the lines it touches first: for data read once
// per pass (a matrix streamed every step), so that it does not push data that
// is read again (the vectors other rows gather) out of L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy()
{
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// bulk_load with an L2 cache policy.
__device__ __forceinline__ void bulk_load_hint(void *dst, const void *src, unsigned bytes, uint64_t *bar,
                                               uint64_t policy)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// Prefetch of `bytes` (multiple of 16, 16-byte aligned) from global memory
// into L2; no completion to wait for.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, unsigned bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Orders this thread's earlier generic-proxy accesses (and the data it has
// acquired from other threads) before its later async-proxy accesses: global
// data written by other CTAs earlier in the same launch, and shared buffers
// just read, before a bulk copy reads or overwrites them.
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace simall
