// pbg_tc.cuh -- fifth-generation tensor cores (tcgen05) for the learned
// traversal ordering: BF16 operands in shared memory, FP32 accumulators in
// tensor memory (TMEM).
//
// Operand layout: K-major, no swizzle.  A tile of R rows x K columns of bf16
// is a grid of 8x8 "core matrices" (8 rows x 16 bytes, 128 contiguous
// bytes); element (r, k) sits at
//     ((r/8) * (K/8) + k/8) * 128 + (r%8) * 16 + (k%8) * 2
// so neighbouring core matrices along K are 128 bytes apart (the leading
// byte offset) and neighbouring 8-row groups are K*16 bytes apart (the
// stride byte offset).  One tcgen05.mma of kind::f16 consumes K = 16, i.e.
// two core matrices along K; the next K step starts 256 bytes further.
//
// Protocol per GEMM: threads write operands (generic proxy) -> fence.proxy.async
// -> __syncthreads -> one thread issues the MMAs and tcgen05.commit to an
// mbarrier -> every thread waits on the mbarrier (bounded) ->
// tcgen05.fence::after_thread_sync -> warps read their 32-lane quarter of the
// accumulator with tcgen05.ld.  TMEM is allocated by warp 0 at kernel start
// and freed before the kernel returns on every path.
#pragma once
#include <cstdint>

#include "pbg_tma.cuh"

namespace pbg {

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t core_offset(int r, int k, int K) {
    return (uint32_t)((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor (K-major, no swizzle, sm_100 format).
__device__ __forceinline__ uint64_t smem_desc(const void* base, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((smem_addr(base) >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor: D = F32, A = B = BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Warp-wide TMEM allocation / release (ncols: power of two, >= 32).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape: the
// warp reads lanes 32*(warp%4) .. +31, one lane per thread).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ uint16_t f2bf(float x) {
    // round to nearest even (inputs here are finite)
    uint32_t u = __float_as_uint(x);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

#endif  // __CUDACC__

}  // namespace pbg
