// 1-D bulk copies global -> shared memory (cp.async.bulk, the TMA engine's
// untiled form) completing on a shared-memory mbarrier, with bounded waits.
//
// Rules the callers keep: source and destination 16-byte aligned, size a
// multiple of 16 bytes; one mbarrier per independent copy group, initialised
// by one thread and made visible to the async proxy before the first copy.
#pragma once

#include <stdint.h>

namespace erp {

// Tries of mbarrier.try_wait before a wait gives up (each try may suspend the
// warp for a short, implementation-defined time; the limit is seconds).
constexpr uint32_t kWaitTries = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (bulk copy) proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
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

// Wait for the barrier phase with the given parity to complete; false once
// `tries` tries (kWaitTries unless given) have run out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t tries = kWaitTries) {
    for (uint32_t i = 0; i < tries; ++i)
        if (mbar_try(bar, parity)) return true;
    return false;
}

}  // namespace erp
