// pbg_tma.cuh -- bulk (TMA) copies into shared memory with mbarrier
// completion, and bounded waits.
//
// Tiles of triangle records are contiguous in global memory, so the 1-D bulk
// form cp.async.bulk suffices: source and destination 16-byte aligned, size a
// multiple of 16 bytes (TriRec is 48 bytes, so every tile qualifies).
// Every wait is bounded: after kSpinLimit polls it records a status word in
// global memory and the caller leaves the kernel; no wait can hang the GPU.
#pragma once
#include <cstdint>

namespace pbg {

constexpr uint32_t kSpinLimit = 1u << 24;

// Device status words (global int[4]); [0] = timeout count, [1] = queue or
// stack overflows, [2] = a shadow batch's origins differ from the kept order's.
enum : int { kStatusTimeout = 0, kStatusOverflow = 1, kStatusOriginMoved = 2 };

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
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

// Bounded wait for phase `parity` of `bar`.  Returns false (and bumps the
// timeout status word) if the phase did not complete within kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status) {
    for (uint32_t i = 0; i < kSpinLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    if (status) atomicAdd(&status[kStatusTimeout], 1);
    return false;
}

}  // namespace pbg
