// nt2g_async.cuh -- bulk copies from global to shared memory on the async
// copy engine (cp.async.bulk), completed on an mbarrier's transaction count,
// and the bounded waits around them.
//
// Every wait polls a limited number of times: a kernel that gives up counts
// the timeout in its translation unit's device counter (nt2g_wait_timeouts
// sums them), waits -- again a limited number of times -- for its own copies
// still in flight, and returns, so no block ever spins forever.
#pragma once
#include "nt2g_common.cuh"

namespace nt2g {

// Polls of one bounded wait.  A poll may suspend the thread for a short,
// system-defined time, so this is far beyond any copy's latency.
constexpr uint32_t kWaitPolls = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// The initialised barriers made visible to the async proxy (the copy engine).
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// This thread's earlier generic-proxy accesses of shared memory ordered
// before its later async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One arrival that also expects `bytes` more of copy transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n"
        "  .reg .pred p;\n"
        "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "  selp.u32 %0, 1, 0, p;\n"
        "}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Wait for the barrier's phase of the given parity; false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit = kWaitPolls)
{
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// `bytes` (a multiple of 16) from 16-byte-aligned global `src` to
// 16-byte-aligned shared `dst`, counted against bar's transactions.  The
// CTA's own shared address is a valid shared::cluster address.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

}  // namespace nt2g
