// pbg_naive.cu -- Accelerator "naive": every ray against every triangle.
//
// Replaces the fork's all-pairs OpenCL kernels (bin/cl/naive.cl:4-231, one
// thread per triangle looping over rays, racing on tHit; bin/cl/naive2.cl,
// one thread per ray) and their host side (accelerators/naive.cpp:204-437).
// Results follow pbrt's CPU test exactly instead of those kernels' widened
// epsilons (naive.cl:2, :32, :38).
//
// Layout: one thread per ray, 256 rays per CTA; the triangle range is split
// across gridDim.y so that small batches still fill 152 SMs.  Triangle tiles
// (128 records, 6 KB) stream into shared memory by bulk TMA copies, two
// stages deep, and every thread reads each record as a broadcast.  With one
// split the thread writes its hit directly; with several, the splits merge
// through a 64-bit atomicMax on (t, index) keys and a finalize pass recomputes
// b1/b2 of the winner with the exact test.  Any-hit: a warp leaves a tile
// once all its rays are occluded, the CTA leaves the tile loop once every
// ray of the CTA is.
#include "pbg_count.cuh"
#include "pbg_internal.h"
#include "pbg_tma.cuh"

namespace pbg {

constexpr int kNaiveThreads = 256;
constexpr int kNaiveTile = 128;
constexpr int kNaiveStages = 2;

// STATS: the counting variant (profiling level 2) adds each thread's filter
// tests, second-stage filter passes, exact tests and exact hits to wcount.
template <bool ANY, bool STATS>
__global__ void __launch_bounds__(kNaiveThreads)
    naive_kernel(const TriRec* __restrict__ tris, int64_t ntri, int64_t per_split,
                 const float4* __restrict__ ro, const float4* __restrict__ rd,
                 const uint8_t* __restrict__ valid, int64_t n, int32_t* __restrict__ prim_out,
                 float* __restrict__ t_out, float* __restrict__ b1_out,
                 float* __restrict__ b2_out, unsigned long long* __restrict__ keys,
                 uint8_t* __restrict__ occ, int* status, unsigned long long* wcount) {
    __shared__ __align__(128) TriRec tile[kNaiveStages][kNaiveTile];
    __shared__ __align__(8) uint64_t bar[kNaiveStages];

    const int64_t ray = (int64_t)blockIdx.x * kNaiveThreads + threadIdx.x;
    const int64_t t0 = (int64_t)blockIdx.y * per_split;
    const int64_t t1 = min(ntri, t0 + per_split);
    const int ntiles = t1 > t0 ? (int)((t1 - t0 + kNaiveTile - 1) / kNaiveTile) : 0;
    const bool split = gridDim.y > 1;

    const bool active = ray < n && (valid == nullptr || valid[ray] != 0);
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
    if (active) {
        o = ro[ray];
        d = rd[ray];
    }
    const float nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    float best_t = d.w, bb1 = 0.f, bb2 = 0.f;
    int32_t best = -1;
    bool done = !active;
    WorkCount wc;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kNaiveStages; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();

    auto issue = [&](int k, int s) {
        const int64_t first = t0 + (int64_t)k * kNaiveTile;
        const uint32_t bytes = (uint32_t)(min((int64_t)kNaiveTile, t1 - first) * sizeof(TriRec));
        mbar_arrive_expect_tx(&bar[s], bytes);
        bulk_g2s(&tile[s][0], tris + first, bytes, &bar[s]);
    };
    if (threadIdx.x == 0)
        for (int k = 0; k < kNaiveStages && k < ntiles; ++k) issue(k, k);

    bool failed = false;
    for (int k = 0; k < ntiles; ++k) {
        const int s = k % kNaiveStages;
        const uint32_t parity = (uint32_t)(k / kNaiveStages) & 1u;
        // a wait that gave up ends the loop for the whole CTA at once, so
        // that no thread is left at a barrier or warp vote below
        const bool ok = mbar_wait_bounded(&bar[s], parity, status);
        if (__syncthreads_or(ok ? 0 : 1)) {
            failed = true;
            break;
        }
        const int cnt = (int)min((int64_t)kNaiveTile, t1 - (t0 + (int64_t)k * kNaiveTile));
        if (ANY) {
            // Every lane runs every iteration (a finished lane skips the
            // test) so that the warp stays converged: a per-lane break out
            // of this loop left lanes running it one small group at a time.
            // The warp leaves once all its rays are occluded.
            if (!__all_sync(0xffffffffu, done)) {
                for (int j = 0; j < cnt; ++j) {
                    if (!done) {
                        const TriRec tr = tile[s][j];
                        if (STATS) wc.filt++;
                        if (pbg_filter(tr, o, d, nd, best_t, STATS ? &wc.filt2 : nullptr)) {
                            float tt, u1, u2;
                            if (STATS) wc.exact++;
                            if (pbg_exact_rec(tr, o, d, best_t, &tt, &u1, &u2)) {
                                if (STATS) wc.hit++;
                                best = __float_as_int(tr.c.w);
                                done = true;
                            }
                        }
                    }
                    if ((j & 7) == 7 && __all_sync(0xffffffffu, done)) break;
                }
            }
        } else if (!done) {
            for (int j = 0; j < cnt; ++j) {
                const TriRec tr = tile[s][j];
                if (STATS) wc.filt++;
                if (!pbg_filter(tr, o, d, nd, best_t, STATS ? &wc.filt2 : nullptr)) continue;
                float tt, u1, u2;
                if (STATS) wc.exact++;
                if (!pbg_exact_rec(tr, o, d, best_t, &tt, &u1, &u2)) continue;
                if (STATS) wc.hit++;
                const int32_t id = __float_as_int(tr.c.w);
                if (tt < best_t || id > best) {
                    best_t = tt;
                    best = id;
                    bb1 = u1;
                    bb2 = u2;
                }
            }
        }
        // Every thread is done with stage s before it is refilled.
        const int all_done = __syncthreads_and(done ? 1 : 0);
        if (ANY && all_done) {
            // Drain the copies already in flight before the CTA leaves.
            if (threadIdx.x == 0)
                for (int q = k + 1; q < ntiles && q < k + kNaiveStages; ++q)
                    mbar_wait_bounded(&bar[q % kNaiveStages],
                                      (uint32_t)(q / kNaiveStages) & 1u, status);
            break;
        }
        if (threadIdx.x == 0 && k + kNaiveStages < ntiles) {
            fence_proxy_async_smem();
            issue(k + kNaiveStages, s);
        }
    }
    if (STATS) wc.flush(wcount);
    if (failed || ray >= n) return;

    if (ANY) {
        if (split) {
            if (best >= 0) occ[ray] = 1;
        } else {
            occ[ray] = (best >= 0) ? 1 : 0;
        }
        return;
    }
    if (split) {
        if (best >= 0) atomicMax(&keys[ray], hit_key(best_t, best));
        return;
    }
    prim_out[ray] = best;
    t_out[ray] = best >= 0 ? best_t : 0.f;
    b1_out[ray] = best >= 0 ? bb1 : 0.f;
    b2_out[ray] = best >= 0 ? bb2 : 0.f;
}

// Turns merged (t, index) keys into hits; b1/b2 (and t) of the winner come
// from the exact test again, which is deterministic.  pos maps an original
// triangle index to its record (NULL = identity).
__global__ void finalize_keys_kernel(const TriRec* __restrict__ tris, const int32_t* __restrict__ pos,
                                     const float4* __restrict__ ro, const float4* __restrict__ rd,
                                     const unsigned long long* __restrict__ keys, int64_t n,
                                     int32_t* prim, float* t, float* b1, float* b2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    int32_t p = -1;
    float tt = 0.f, u1 = 0.f, u2 = 0.f;
    if (k != 0ull) {
        p = key_prim(k);
        const TriRec tr = tris[pos ? pos[p] : p];
        const float4 o = ro[i], d = rd[i];
        if (!pbg_exact_rec(tr, o, d, d.w, &tt, &u1, &u2)) {
            p = -1;  // unreachable: the key came from this same test
            tt = u1 = u2 = 0.f;
        }
    }
    prim[i] = p;
    t[i] = tt;
    b1[i] = u1;
    b2[i] = u2;
}

int finalize_keys(pbg_scene* s, const int32_t* pos, const float4* o, const float4* d,
                  const unsigned long long* keys, int64_t n, int32_t* prim, float* t, float* b1,
                  float* b2, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    const int threads = 256;
    prof_begin(s, st);
    finalize_keys_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, st>>>(
        (const TriRec*)s->tris.ptr, pos, o, d, keys, n, prim, t, b1, b2);
    prof_end(s, st, kStageOther, 1);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

static int naive_launch_shape(pbg_scene* s, int64_t n, int64_t* per_split, unsigned* splits) {
    const int64_t ray_ctas = (n + kNaiveThreads - 1) / kNaiveThreads;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    // Aim for tune.naive_ctas CTAs per SM (4 unless tuned); never split
    // below one tile per split.
    const int64_t per_sm = s->tune.naive_ctas > 0 ? s->tune.naive_ctas : 4;
    int64_t want = (per_sm * (int64_t)sms + ray_ctas - 1) / ray_ctas;
    int64_t max_splits = (s->ntri + kNaiveTile - 1) / kNaiveTile;
    if (want > max_splits) want = max_splits;
    if (want < 1) want = 1;
    if (want > 65535) want = 65535;
    int64_t per = (s->ntri + want - 1) / want;
    per = ((per + kNaiveTile - 1) / kNaiveTile) * kNaiveTile;
    *per_split = per > 0 ? per : kNaiveTile;
    *splits = (unsigned)((s->ntri + *per_split - 1) / *per_split);
    if (*splits < 1) *splits = 1;
    return PBG_OK;
}

int naive_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                  int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    int64_t per;
    unsigned splits;
    naive_launch_shape(s, n, &per, &splits);
    dim3 grid((unsigned)((n + kNaiveThreads - 1) / kNaiveThreads), splits);
    unsigned long long* keys = nullptr;
    if (splits > 1) {
        int rc = ensure(s->work.keys, (size_t)n * sizeof(unsigned long long));
        if (rc) return rc;
        keys = (unsigned long long*)s->work.keys.ptr;
        PBG_CUDA(cudaMemsetAsync(keys, 0, (size_t)n * sizeof(unsigned long long), st));
    }
    prof_begin(s, st);
    if (s->prof.level >= 2)
        naive_kernel<false, true><<<grid, kNaiveThreads, 0, st>>>(
            (const TriRec*)s->tris.ptr, s->ntri, per, o, d, valid, n, prim, t, b1, b2, keys, nullptr,
            (int*)s->err.ptr, (unsigned long long*)s->workc.ptr);
    else
        naive_kernel<false, false><<<grid, kNaiveThreads, 0, st>>>(
            (const TriRec*)s->tris.ptr, s->ntri, per, o, d, valid, n, prim, t, b1, b2, keys, nullptr,
            (int*)s->err.ptr, nullptr);
    prof_end(s, st, kStageTraverse, 1);
    PBG_CUDA(cudaGetLastError());
    if (splits > 1) return finalize_keys(s, nullptr, o, d, keys, n, prim, t, b1, b2, st);
    return PBG_OK;
}

int naive_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                   uint8_t* occ, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    int64_t per;
    unsigned splits;
    naive_launch_shape(s, n, &per, &splits);
    dim3 grid((unsigned)((n + kNaiveThreads - 1) / kNaiveThreads), splits);
    if (splits > 1) PBG_CUDA(cudaMemsetAsync(occ, 0, (size_t)n, st));
    prof_begin(s, st);
    if (s->prof.level >= 2)
        naive_kernel<true, true><<<grid, kNaiveThreads, 0, st>>>(
            (const TriRec*)s->tris.ptr, s->ntri, per, o, d, valid, n, nullptr, nullptr, nullptr,
            nullptr, nullptr, occ, (int*)s->err.ptr, (unsigned long long*)s->workc.ptr);
    else
        naive_kernel<true, false><<<grid, kNaiveThreads, 0, st>>>(
            (const TriRec*)s->tris.ptr, s->ntri, per, o, d, valid, n, nullptr, nullptr, nullptr,
            nullptr, nullptr, occ, (int*)s->err.ptr, nullptr);
    prof_end(s, st, kStageTraverse, 1);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

}  // namespace pbg
