// pbg_noalloc.cu -- nearest hit for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc at all: code that runs inside another
// framework's memory pool or allocator hooks, a renderer that has already
// committed every byte of the device to its own arenas, or a plug-in whose
// host forbids allocation on its call path.  pbg_intersect_naive_noalloc
// serves them: the caller passes the triangles, the rays and the output
// arrays, all in device memory, and the call allocates nothing.  It runs
// the all-pairs ("naive") test; its only scratch -- the 64-bit (t, index)
// merge key of each ray, 8 MB for the 2^20-ray maximum -- lives in one
// file-scope __device__ array, which every GPU that loads this library holds
// until the process exits.
//
// Limits and rules:
//   - at most kNoallocMaxRays rays per call (larger batches are rejected);
//   - every call shares the one array, so calls that overlap on the GPU
//     (different streams, or different host threads on one device) race;
//     serialise them;
//   - every call looks up the array's device address with
//     cudaGetSymbolAddress in the calling thread's current context (after
//     the first call in a context that is a host-side table lookup), so a
//     device reset, or a caller on its own driver-API context, gets the
//     address that is valid there; the first call in each context loads the
//     library's device code and should come before any stream capture;
//   - the rays (o4, d4) must be 16-byte aligned and the other arrays 4-byte
//     aligned (misaligned views are rejected, not faulted on).
#include <cstdint>

#include "pbg_internal.h"
#include "pbg_tma.cuh"

namespace pbg {

constexpr int64_t kNoallocMaxRays = 1 << 20;
constexpr size_t kNoallocBytes = (size_t)kNoallocMaxRays * sizeof(unsigned long long);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kNaThreads = 256;
constexpr int kNaTile = 128;

// Triangle records built in shared memory from the caller's v0 v1 v2 floats,
// with e1 = p2 - p1 and e2 = p3 - p1 rounded as pbrt rounds them.
__device__ __forceinline__ TriRec rec_from_tri9(const float* v, int32_t index) {
    const float e1x = __fsub_rn(v[3], v[0]), e1y = __fsub_rn(v[4], v[1]), e1z = __fsub_rn(v[5], v[2]);
    const float e2x = __fsub_rn(v[6], v[0]), e2y = __fsub_rn(v[7], v[1]), e2z = __fsub_rn(v[8], v[2]);
    TriRec r;
    r.a = make_float4(v[0], v[1], v[2], fabsf(e1x) + fabsf(e1y) + fabsf(e1z));
    r.b = make_float4(e1x, e1y, e1z, fabsf(e2x) + fabsf(e2y) + fabsf(e2z));
    r.c = make_float4(e2x, e2y, e2z, __int_as_float(index));
    return r;
}

__global__ void __launch_bounds__(kNaThreads)
    noalloc_naive_kernel(const float* __restrict__ tri9, int64_t ntri, int64_t per_split,
                         const float4* __restrict__ ro, const float4* __restrict__ rd, int64_t n,
                         unsigned long long* __restrict__ keys) {
    __shared__ TriRec tile[kNaTile];
    __shared__ float raw[kNaTile * 9];
    const int64_t ray = (int64_t)blockIdx.x * kNaThreads + threadIdx.x;
    const int64_t t0 = (int64_t)blockIdx.y * per_split;
    const int64_t t1 = min(ntri, t0 + per_split);
    const bool active = ray < n;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
    if (active) {
        o = ro[ray];
        d = rd[ray];
    }
    const float nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    float best_t = d.w;
    int32_t best = -1;
    for (int64_t base = t0; base < t1; base += kNaTile) {
        const int cnt = (int)min((int64_t)kNaTile, t1 - base);
        __syncthreads();
        // the tile's vertices in one coalesced sweep, then the records
        const float* src = tri9 + 9 * base;
        for (int k = threadIdx.x; k < 9 * cnt; k += kNaThreads) raw[k] = src[k];
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kNaThreads) tile[k] = rec_from_tri9(raw + 9 * k, (int32_t)(base + k));
        __syncthreads();
        if (!active) continue;
        for (int j = 0; j < cnt; ++j) {
            const TriRec tr = tile[j];
            if (!pbg_filter(tr, o, d, nd, best_t)) continue;
            float tt, u1, u2;
            if (!pbg_exact_rec(tr, o, d, best_t, &tt, &u1, &u2)) continue;
            const int32_t id = __float_as_int(tr.c.w);
            if (tt < best_t || id > best) {
                best_t = tt;
                best = id;
            }
        }
    }
    if (active && best >= 0) atomicMax(&keys[ray], hit_key(best_t, best));
}

__global__ void noalloc_finalize_kernel(const float* __restrict__ tri9, const float4* __restrict__ ro,
                                        const float4* __restrict__ rd,
                                        const unsigned long long* __restrict__ keys, int64_t n,
                                        int32_t* prim, float* t, float* b1, float* b2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    int32_t p = -1;
    float tt = 0.f, u1 = 0.f, u2 = 0.f;
    if (k != 0ull) {
        p = key_prim(k);
        const TriRec tr = rec_from_tri9(tri9 + 9 * (int64_t)p, p);
        const float4 o = ro[i], d = rd[i];
        if (!pbg_exact_rec(tr, o, d, d.w, &tt, &u1, &u2)) {
            p = -1;
            tt = u1 = u2 = 0.f;
        }
    }
    prim[i] = p;
    t[i] = tt;
    b1[i] = u1;
    b2[i] = u2;
}

// Device address of the scratch array in the current context.  Looked up on
// every call: a cached address would outlive a device reset, and would be
// wrong for a caller that runs on another context of the same device.
static unsigned char* noalloc_scratch(int* status) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        *status = cuda_status(e, "cudaGetSymbolAddress(noalloc scratch)");
        return nullptr;
    }
    *status = PBG_OK;
    return (unsigned char*)p;
}

}  // namespace pbg

using namespace pbg;

extern "C" int pbg_intersect_naive_noalloc(const float* tri9, int64_t ntri, const float* o4,
                                           const float* d4, int64_t n, int32_t* prim, float* t,
                                           float* b1, float* b2, void* stream) {
    if (n < 0 || ntri < 0 || ntri > (int64_t)INT32_MAX / 2 || (ntri > 0 && !tri9) ||
        (n > 0 && (!o4 || !d4 || !prim || !t || !b1 || !b2))) {
        set_last_error("pbg_intersect_naive_noalloc: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (n > kNoallocMaxRays) {
        set_last_error("pbg_intersect_naive_noalloc: more than 1048576 rays in one call "
                       "(the fixed scratch holds one merge key per ray)");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    const uintptr_t a16 = (uintptr_t)o4 | (uintptr_t)d4;
    const uintptr_t a4 = (uintptr_t)tri9 | (uintptr_t)prim | (uintptr_t)t | (uintptr_t)b1 | (uintptr_t)b2;
    if ((a16 & 15u) || (a4 & 3u)) {
        set_last_error("pbg_intersect_naive_noalloc: o4/d4 must be 16-byte aligned, the other arrays 4-byte "
                       "aligned");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PBG_OK;
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    int rc = PBG_OK;
    unsigned char* scratch = noalloc_scratch(&rc);
    if (!scratch) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long* keys = (unsigned long long*)scratch;
    // the array keeps the previous call's keys: clear this call's range
    PBG_CUDA(cudaMemsetAsync(keys, 0, (size_t)n * sizeof(unsigned long long), st));
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int64_t ray_ctas = (n + kNaThreads - 1) / kNaThreads;
    int64_t splits = (4 * (int64_t)sms + ray_ctas - 1) / ray_ctas;
    const int64_t max_splits = (ntri + kNaTile - 1) / kNaTile;
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    const int64_t per = ((ntri + splits - 1) / splits + kNaTile - 1) / kNaTile * kNaTile;
    splits = per > 0 ? (ntri + per - 1) / per : 1;
    if (splits < 1) splits = 1;
    if (ntri > 0) {
        dim3 grid((unsigned)ray_ctas, (unsigned)splits);
        noalloc_naive_kernel<<<grid, kNaThreads, 0, st>>>(tri9, ntri, per > 0 ? per : kNaTile,
                                                          (const float4*)o4, (const float4*)d4, n, keys);
        PBG_CUDA(cudaGetLastError());
    }
    noalloc_finalize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        tri9, (const float4*)o4, (const float4*)d4, keys, n, prim, t, b1, b2);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}
