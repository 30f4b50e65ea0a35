// bulk_copy.cuh -- Blackwell bulk asynchronous copies (the TMA engine's
// non-tensor form, cp.async.bulk) into shared memory, completed on an
// mbarrier, with bounded waits.
//
// Rules kept by every caller:
//   * source and destination 16-byte aligned, size a multiple of 16 bytes
//     and below 2^20 per barrier phase (mbarrier transaction count);
//   * a wait gives up after max_spin polls and reports it, so a copy that
//     never lands cannot hang the GPU; the caller then drains its other
//     copies (again bounded) before it returns.
#pragma once

#include <stdint.h>

namespace ucfd {
namespace dev {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the asynchronous (copy) proxy.
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later asynchronous-proxy writes to it (buffer reuse).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One arrival that also announces the bytes the phase waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Global -> shared bulk copy; its bytes complete the barrier's transaction.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Asks L2 to fetch [src, src + bytes) (16-byte aligned, multiple of 16);
// no completion to wait for.
__device__ __forceinline__ void prefetch_l2_bulk(const void *src, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete; false after
// max_spin unsuccessful polls (each poll may suspend the thread briefly).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, long long max_spin) {
    for (long long i = 0; i < max_spin; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

}  // namespace dev
}  // namespace ucfd
