// pbg_tune.cu -- launch-shape autotuner for one scene and one batch shape.
//
// The reference exposes its launch shapes as scene-file parameters
// (rayhierarchy.cpp:1329-1348: chunkXSize, chunkYSize, height; the work-group
// sizes of its OpenCL kernels are fixed in GPUparallel.cpp).  Here the
// leaves are one warp of 32 rays by construction, and the shapes that can
// vary without changing any result are tuned per scene on a sample batch:
//   naive         CTAs per SM that the triangle splits aim for: 2, 4, 8, 16
//   rayhierarchy  nodes of the level the descent is seeded at (64, 256,
//                 1024) x CTAs per SM of the grid-stride kernels (16, 32),
//                 kept apart for nearest-hit and any-hit batches
//   ray-bvh       the walk for this batch class (any-hit or not, coherent
//                 or not): one thread per ray, persistent warps, warp
//                 packets over the ray hierarchy's leaves (sorted) or over
//                 the batch in its own order, or persistent warps over the
//                 eight-wide tree (with the warp's triangle tests spread over
//                 its lanes or not); skipped when pbg_params.walk fixes the
//                 walk
// Every candidate traces the same batch; its results must equal the first
// candidate's bit for bit (prim, t, b1, b2 of hits, or occlusion), else the
// call fails with PBG_ERR_INTERNAL and the scene keeps its previous shapes.
// The fastest candidate (CUDA events on the caller's stream, best of `reps`
// after one warm-up run) becomes the scene's setting.
#include <algorithm>
#include <cstring>
#include <vector>

#include "pbg_internal.h"

namespace pbg {

__global__ void tune_compare_hits_kernel(const int32_t* __restrict__ p0, const float* __restrict__ t0,
                                         const float* __restrict__ u0, const float* __restrict__ v0,
                                         const int32_t* __restrict__ p1, const float* __restrict__ t1,
                                         const float* __restrict__ u1, const float* __restrict__ v1,
                                         int64_t n, unsigned long long* mismatches) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool same = p0[i] == p1[i];
    if (same && p0[i] >= 0)
        same = __float_as_uint(t0[i]) == __float_as_uint(t1[i]) &&
               __float_as_uint(u0[i]) == __float_as_uint(u1[i]) &&
               __float_as_uint(v0[i]) == __float_as_uint(v1[i]);
    if (!same) atomicAdd(mismatches, 1ull);
}

__global__ void tune_compare_bytes_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                          int64_t n, unsigned long long* mismatches) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && a[i] != b[i]) atomicAdd(mismatches, 1ull);
}

namespace {

struct Candidate {
    int v[3];
};

void apply(pbg_scene* s, int any, int incoherent, const Candidate& c) {
    switch (s->accel) {
        case PBG_ACCEL_NAIVE: s->tune.naive_ctas = c.v[0]; break;
        case PBG_ACCEL_RAYHIERARCHY:
            s->tune.rh_seed[any] = c.v[0];
            s->tune.rh_grid[any] = c.v[1];
            break;
        case PBG_ACCEL_RAYBVH: s->tune.bvh_walk[any][incoherent] = c.v[0]; break;
    }
}

Candidate current(const pbg_scene* s, int any, int incoherent) {
    Candidate c{{0, 0, 0}};
    switch (s->accel) {
        case PBG_ACCEL_NAIVE: c.v[0] = s->tune.naive_ctas; break;
        case PBG_ACCEL_RAYHIERARCHY:
            c.v[0] = s->tune.rh_seed[any];
            c.v[1] = s->tune.rh_grid[any];
            break;
        case PBG_ACCEL_RAYBVH: c.v[0] = s->tune.bvh_walk[any][incoherent]; break;
    }
    return c;
}

std::vector<Candidate> candidates(const pbg_scene* s) {
    std::vector<Candidate> out;
    switch (s->accel) {
        case PBG_ACCEL_NAIVE:
            for (int k : {4, 2, 8, 16}) out.push_back({{k, 0, 0}});
            break;
        case PBG_ACCEL_RAYHIERARCHY:
            for (int seed : {256, 64, 1024})
                for (int grid : {32, 16}) out.push_back({{seed, grid, 0}});
            break;
        case PBG_ACCEL_RAYBVH:
            if (s->params.walk != 0) {
                out.push_back({{s->params.walk, 0, 0}});
            } else {
                out.push_back({{1, 0, 0}});
                out.push_back({{2, 0, 0}});
                out.push_back({{3, 0, 0}});
                out.push_back({{4, 0, 0}});
                out.push_back({{5, 0, 0}});
                out.push_back({{6, 0, 0}});
            }
            break;
    }
    return out;
}

}  // namespace
}  // namespace pbg

using namespace pbg;

extern "C" int pbg_autotune(pbg_scene* s, const float* o4, const float* d4, const uint8_t* valid, int64_t n,
                            int32_t query, int32_t reps, pbg_tune_result* out, void* stream) {
    if (!s || !out || n <= 0 || !o4 || !d4 || (query & ~3) != 0 ||
        ((uintptr_t)o4 & 15u) != 0 || ((uintptr_t)d4 & 15u) != 0) {
        set_last_error("pbg_autotune: bad arguments (device rays 16-byte aligned, n > 0, query 0-3)");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    memset(out, 0, sizeof(*out));
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    const int any = query & 1, incoherent = (query >> 1) & 1;
    if (reps < 1) reps = 3;
    const std::vector<Candidate> cand = candidates(s);
    const Candidate before = current(s, any, incoherent);
    const int saved_hint = s->walk_hint;
    const float4* o = (const float4*)o4;
    const float4* d = (const float4*)d4;

    // results of the first candidate (reference) and of the one being timed
    DeviceBuffer ref, cur, mism;
    const size_t per_ray = any ? 1 : 16;
    int rc = PBG_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto fail = [&](int code) {
        apply(s, any, incoherent, before);
        s->walk_hint = saved_hint;
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        release(ref);
        release(cur);
        release(mism);
        return code;
    };
    if ((rc = ensure(ref, (size_t)n * per_ray)) || (rc = ensure(cur, (size_t)n * per_ray)) ||
        (rc = ensure(mism, sizeof(unsigned long long))))
        return fail(rc);
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return fail(cuda_status(cudaGetLastError(), "cudaEventCreate"));

    auto run = [&](DeviceBuffer& buf) {
        if (s->accel == PBG_ACCEL_RAYBVH) s->walk_hint = incoherent;
        if (any) return run_occluded(s, o, d, valid, n, (uint8_t*)buf.ptr, st);
        int32_t* prim = (int32_t*)buf.ptr;
        float* t = (float*)(prim + n);
        return run_nearest(s, o, d, valid, n, prim, t, t + n, t + 2 * n, st);
    };

    const int nc = (int)std::min<size_t>(cand.size(), 16);
    float best_ms = 0.f;
    int best = -1;
    for (int k = 0; k < nc; ++k) {
        apply(s, any, incoherent, cand[k]);
        DeviceBuffer& dst = k == 0 ? ref : cur;
        if ((rc = run(dst))) return fail(rc);  // warm-up (and the compared result)
        float ms = 0.f;
        for (int r = 0; r < reps; ++r) {
            cudaEventRecord(e0, st);
            if ((rc = run(dst))) return fail(rc);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                return fail(cuda_status(cudaGetLastError(), "cudaEventSynchronize"));
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            ms = r == 0 ? t : std::min(ms, t);
        }
        if ((rc = check_device_status(s, st))) return fail(rc);
        if (k > 0) {
            unsigned long long* mm = (unsigned long long*)mism.ptr;
            if (cudaMemsetAsync(mm, 0, sizeof(*mm), st) != cudaSuccess)
                return fail(cuda_status(cudaGetLastError(), "cudaMemsetAsync"));
            const unsigned blocks = (unsigned)((n + 255) / 256);
            if (any) {
                tune_compare_bytes_kernel<<<blocks, 256, 0, st>>>((const uint8_t*)ref.ptr,
                                                                  (const uint8_t*)cur.ptr, n, mm);
            } else {
                const int32_t* p0 = (const int32_t*)ref.ptr;
                const int32_t* p1 = (const int32_t*)cur.ptr;
                const float* f0 = (const float*)(p0 + n);
                const float* f1 = (const float*)(p1 + n);
                tune_compare_hits_kernel<<<blocks, 256, 0, st>>>(p0, f0, f0 + n, f0 + 2 * n, p1, f1, f1 + n,
                                                                 f1 + 2 * n, n, mm);
            }
            unsigned long long h = 0;
            if (cudaMemcpyAsync(&h, mm, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return fail(cuda_status(cudaGetLastError(), "autotune compare"));
            out->mismatches += h;
            if (h != 0) {
                set_last_error("pbg_autotune: a launch shape changed the results");
                return fail(PBG_ERR_INTERNAL);
            }
        }
        for (int j = 0; j < 3; ++j) out->setting[k][j] = cand[k].v[j];
        out->ms[k] = ms;
        if (best < 0 || ms < best_ms) {
            best = k;
            best_ms = ms;
        }
    }
    out->ncandidates = nc;
    out->best = best;
    apply(s, any, incoherent, cand[best]);
    s->walk_hint = saved_hint;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release(ref);
    release(cur);
    release(mism);
    return PBG_OK;
}
