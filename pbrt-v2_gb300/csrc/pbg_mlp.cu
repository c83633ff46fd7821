// pbg_mlp.cu -- tensor-core (tcgen05) kernels of the learned traversal
// ordering: a generic BF16 GEMM with FP32 accumulation in TMEM (the training
// passes are built from it) and, in pbg_learn.cu, the fused inference MLP.
#include <mutex>

#include "pbg_internal.h"
#include "pbg_tc.cuh"

namespace pbg {

constexpr int kTcRows = 128;   // M of one MMA (cta_group::1)
constexpr int kTcKChunk = 128; // K staged per round

// C[M x N] (+)= A[M x K] * B[N x K]^T.  A, B: row-major bf16 (K contiguous,
// i.e. K-major); C: row-major fp32.  M % 128 == 0, N % 16 == 0 and
// 16 <= N <= 256, K % 16 == 0.  One CTA of 4 warps per 128-row tile and
// K slice: blockIdx.y takes K chunks [y * kslice, (y + 1) * kslice); with
// more than one slice each CTA writes its partial product to
// work[y][M][N] and tc_reduce_kernel sums the slices in order (split-K for
// the weight gradients, whose K is the batch).
__global__ void __launch_bounds__(128)
    tc_gemm_kernel(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B, float* __restrict__ C,
                   int M, int N, int K, int accumulate_c, int* status, int kslice, float* __restrict__ work) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sa = smem;                                 // 128 x 128 bf16 = 32 KB
    uint8_t* sb = smem + kTcRows * kTcKChunk * 2;       // 256 x 128 bf16 = 64 KB
    uint64_t* bar = (uint64_t*)(sb + 256 * kTcKChunk * 2);
    uint32_t* tslot = (uint32_t*)(bar + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kTcRows;
    uint32_t ncols = 32;
    while ((int)ncols < N) ncols <<= 1;
    if (warp == 0) tmem_alloc(tslot, ncols);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    uint32_t phase = 0;
    bool ok = true;
    const int kbeg = blockIdx.y * kslice, kend = min(K, kbeg + kslice);
    for (int k0 = kbeg; k0 < kend && ok; k0 += kTcKChunk) {
        const int kc = min(kTcKChunk, kend - k0);
        const int kb = kc >> 3;  // 16-byte groups per row
        for (int idx = threadIdx.x; idx < kTcRows * kb; idx += blockDim.x) {
            const int r = idx / kb, g = idx % kb;
            const uint4 v = *(const uint4*)(A + (size_t)(m0 + r) * K + k0 + g * 8);
            *(uint4*)(sa + core_offset(r, g * 8, kc)) = v;
        }
        for (int idx = threadIdx.x; idx < N * kb; idx += blockDim.x) {
            const int r = idx / kb, g = idx % kb;
            const uint4 v = *(const uint4*)(B + (size_t)r * K + k0 + g * 8);
            *(uint4*)(sb + core_offset(r, g * 8, kc)) = v;
        }
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (threadIdx.x == 0) {
            const uint32_t sbo = (uint32_t)kb * 128u;
            for (int ks = 0; ks < (kc >> 4); ++ks) {
                const uint64_t ad = smem_desc(sa + ks * 256, 128u, sbo);
                const uint64_t bd = smem_desc(sb + ks * 256, 128u, sbo);
                tc_mma(tbase, ad, bd, idesc_bf16(kTcRows, N), (k0 > kbeg || ks > 0) ? 1u : 0u);
            }
            tc_commit(bar);
        }
        ok = mbar_wait_bounded(bar, phase, status);
        phase ^= 1u;
        tc_fence_after();
    }
    if (ok) {
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (kbeg >= kend)  // an empty K slice contributes nothing
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = 0.f;
            if (gridDim.y > 1) {
                float* out = work + ((size_t)blockIdx.y * M + row) * N + c0;
#pragma unroll
                for (int j = 0; j < 16; ++j) out[j] = v[j];
            } else {
                float* out = C + (size_t)row * N + c0;
#pragma unroll
                for (int j = 0; j < 16; ++j) out[j] = accumulate_c ? out[j] + v[j] : v[j];
            }
        }
    } else if (threadIdx.x == 0) {
        // give in-flight MMAs one more bounded window before TMEM is released
        mbar_wait_bounded(bar, phase ^ 1u, status);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tbase, ncols);
}

// C (+)= the sum of the K slices' partial products, slice by slice.
__global__ void tc_reduce_kernel(const float* __restrict__ work, int slices, int64_t mn,
                                 float* __restrict__ C, int accumulate_c) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mn) return;
    float acc = accumulate_c ? C[i] : 0.f;
    for (int y = 0; y < slices; ++y) acc += work[(int64_t)y * mn + i];
    C[i] = acc;
}

size_t tc_gemm_smem_bytes() { return (size_t)kTcRows * kTcKChunk * 2 + 256 * kTcKChunk * 2 + 64; }

// K slices for a GEMM given a split-K workspace: powers of two, at most one
// per K chunk, about one CTA per SM in all.
int tc_gemm_slices(int M, int K) {
    const int tiles = M / kTcRows, chunks = (K + kTcKChunk - 1) / kTcKChunk;
    int slices = 1;
    while (slices * 2 <= chunks && tiles * slices * 2 <= 152) slices *= 2;
    return slices;
}

size_t tc_gemm_work_floats(int M, int N, int K) {
    return (size_t)tc_gemm_slices(M, K) * (size_t)M * (size_t)N;
}

int tc_gemm(const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K, int accumulate,
            int* status, cudaStream_t st, float* work) {
    if (M <= 0 || M % kTcRows || N < 16 || N > 256 || N % 16 || K <= 0 || K % 16) {
        set_last_error("tc_gemm: M % 128, 16 <= N <= 256 with N % 16, K % 16 required");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    // a per-device setting (cheap, idempotent): set on every call so that each
    // device the library launches on has it
    PBG_CUDA(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_gemm_smem_bytes()));
    const int slices = work ? tc_gemm_slices(M, K) : 1;
    const int chunks = (K + kTcKChunk - 1) / kTcKChunk;
    const int kslice = ((chunks + slices - 1) / slices) * kTcKChunk;
    tc_gemm_kernel<<<dim3(M / kTcRows, slices), 128, tc_gemm_smem_bytes(), st>>>(
        A, B, C, M, N, K, accumulate, status, kslice, work);
    PBG_CUDA(cudaGetLastError());
    if (slices > 1) {
        const int64_t mn = (int64_t)M * N;
        tc_reduce_kernel<<<(unsigned)((mn + 255) / 256), 256, 0, st>>>(work, slices, mn, C, accumulate);
        PBG_CUDA(cudaGetLastError());
    }
    return PBG_OK;
}

}  // namespace pbg

using namespace pbg;

// Status words for library-level launches that have no scene, one block per
// device (allocated on that device the first time it is used).
static int* g_status[64] = {nullptr};
static std::mutex g_status_mu;

extern "C" int pbg_tc_gemm_bf16(const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t N,
                                int32_t K, int32_t accumulate, void* stream) {
    if (!A || !B || !C) {
        pbg::set_last_error("pbg_tc_gemm_bf16: null pointer");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        pbg::set_last_error("pbg_tc_gemm_bf16: no current CUDA device");
        return PBG_ERR_NO_DEVICE;
    }
    int* status = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_status_mu);
        if (!g_status[dev]) {
            cudaError_t e = cudaMalloc(&g_status[dev], 4 * sizeof(int));
            if (e != cudaSuccess) return pbg::cuda_status(e, "cudaMalloc(status)");
            cudaMemset(g_status[dev], 0, 4 * sizeof(int));
        }
        status = g_status[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    int rc = pbg::tc_gemm(A, B, C, M, N, K, accumulate, status, st, nullptr);
    if (rc) return rc;
    int h[4] = {0, 0, 0, 0};
    PBG_CUDA(cudaMemcpyAsync(h, status, sizeof(h), cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    if (h[pbg::kStatusTimeout]) {
        cudaMemset(status, 0, 4 * sizeof(int));
        pbg::set_last_error("pbg_tc_gemm_bf16: bounded mbarrier wait expired");
        return PBG_ERR_DEVICE_TIMEOUT;
    }
    return PBG_OK;
}
