// pbg_batch.cu -- many ray-bvh scenes answered by one persistent launch.
//
// The reference answers one scene's batch per call (core/scene.cpp:69-120
// dispatching to accelerators/rayBVH.cpp:615-1323), so a set of small scenes
// leaves most of the device idle between calls.  A scene set keeps every
// scene's BVH nodes and triangle records in two arrays in HBM; one trace call
// answers the nearest-hit and any-hit rays of all scenes with one persistent
// kernel:
//
//  * Work items are tiles of `tile` consecutive rays of one scene and one
//    query kind, numbered scene-major (scene 0 nearest, scene 0 any-hit,
//    scene 1 nearest, ...) so that scenes finish in order instead of all at
//    the end.  A warp takes the next item from a global counter (one atomic
//    per item), finds its segment by binary search over the item offsets and
//    walks each ray with the same per-ray walk as the single-scene ray-bvh
//    kernel (pbg_walk.cuh), so results are bit-identical to it.
//  * When a warp finishes an item it counts down its scene; the warp that
//    finishes the scene's last item stamps %globaltimer, giving per-scene
//    completion times relative to the stamp of the reset kernel.
//  * The reset + trace launch pair is captured once as a CUDA graph and
//    replayed while the caller passes the same arrays and launch shape.
//  * Or, per-lane persistent: every lane refills from a counter over all
//    rays of the set (batch_persistent_kernel) -- better for incoherent
//    rays, whose walks end at very different times; or the same over every
//    scene's eight-wide tree (pbg_wide.cuh), one launch per query kind.
//  * The autotuner times the candidate (walk, tile, CTAs per SM, threads)
//    shapes on the caller's queries and keeps the fastest.
// No kernel here waits on another CTA: the queue is a plain fetch-and-add.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

#include "pbg_internal.h"
#include "pbg_tma.cuh"
#include "pbg_walk.cuh"
#include "pbg_wide.cuh"

namespace pbg {

constexpr int kBatchMaxScenes = 4096;
constexpr int kBatchMaxThreads = 256;

struct SceneDesc {
    const BvhNode* nodes;
    const TriRec* tris;
    int32_t unculled;
    int32_t pad;
    const WideNode* wide;  // the eight-wide tree and its record copy (walks 3 and 4)
    const TriRec* wtris;
};

struct BatchArgs {
    const SceneDesc* scenes;
    int32_t nscenes;
    int32_t tile;
    const int64_t* item_off;  // [2 * nscenes + 1], segment 2k + kind
    const int64_t* ray_off;   // [2 * nscenes]: first ray of each segment
    const int64_t* ray_end;   // [2 * nscenes]
    const int64_t* rseg_off;  // [2 * nscenes + 1]: rays before each segment
    const float4* o4n;
    const float4* d4n;
    int32_t* prim;
    float* t;
    float* b1;
    float* b2;
    const float4* o4s;
    const float4* d4s;
    uint8_t* occ;
    unsigned long long* head;       // queue head
    int32_t* remaining;             // items left per scene
    unsigned long long* done_ns;    // completion stamp per scene
    unsigned long long* start_ns;   // stamp of the reset kernel
    int* status;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    return v;
}

__global__ void batch_reset_kernel(BatchArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) {
        a.head[0] = 0ull;
        a.head[1] = 0ull;  // the any-hit launch of the wide walks
        *a.start_ns = global_ns();
    }
    if (k < a.nscenes) {
        a.remaining[k] = (int32_t)(a.item_off[2 * k + 2] - a.item_off[2 * k]);
        a.done_ns[k] = 0ull;
    }
}

__global__ void __launch_bounds__(kBatchMaxThreads) batch_trace_kernel(BatchArgs a) {
    const int lane = threadIdx.x & 31;
    const int nseg = 2 * a.nscenes;
    const int64_t total = a.item_off[nseg];
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(a.head, 1ull);
        item = __shfl_sync(0xffffffffu, item, 0);
        if ((int64_t)item >= total) break;
        // largest segment with item_off[seg] <= item (empty segments are skipped)
        int lo = 0, hi = nseg;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (a.item_off[mid] <= (int64_t)item) lo = mid;
            else hi = mid;
        }
        const int k = lo >> 1;
        const bool any = (lo & 1) != 0;
        const int64_t first = a.ray_off[lo] + ((int64_t)item - a.item_off[lo]) * a.tile;
        const int64_t end = min(first + (int64_t)a.tile, a.ray_end[lo]);
        const SceneDesc sd = a.scenes[k];
        bool ok = true;
        for (int64_t r = first + lane; r < end; r += 32) {
            WorkCount wc;
            if (any) {
                const float4 o = a.o4s[r], d = a.d4s[r];
                WalkHit h{d.w, 0.f, 0.f, -1};
                ok &= bvh_walk<true, false, false>(sd.nodes, sd.tris, sd.unculled, o, d, INT32_MIN, 0,
                                                   h, wc);
                a.occ[r] = h.prim >= 0 ? 1 : 0;
            } else {
                const float4 o = a.o4n[r], d = a.d4n[r];
                WalkHit h{d.w, 0.f, 0.f, -1};
                ok &= bvh_walk<false, false, false>(sd.nodes, sd.tris, sd.unculled, o, d, INT32_MIN, 0,
                                                    h, wc);
                const bool hit = h.prim >= 0;
                a.prim[r] = h.prim;
                a.t[r] = hit ? h.t : 0.f;
                a.b1[r] = hit ? h.b1 : 0.f;
                a.b2[r] = hit ? h.b2 : 0.f;
            }
        }
        if (!ok) atomicAdd(&a.status[kStatusOverflow], 1);
        __syncwarp();
        if (lane == 0) {
            __threadfence();
            if (atomicSub(&a.remaining[k], 1) == 1) a.done_ns[k] = global_ns();
        }
    }
}

// Per-lane persistent form: a lane takes the next ray of the whole set (all
// scenes' nearest and any-hit rays numbered scene-major) from one counter as
// soon as its ray is done, walks inner nodes until it holds a leaf, and the
// warp tests leaves together (the while-while walk of the single-scene
// persistent kernel, with the scene looked up per ray).  Completion stamps:
// the lanes that finish a ray in an iteration raise their scene's stamp
// with one atomicMax per scene per warp.
// PACK: one 8-byte stack entry (WalkStack) when every scene has fewer than
// 2^24 records.
template <bool PACK>
__global__ void __launch_bounds__(kBatchMaxThreads) batch_persistent_kernel(BatchArgs a) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int nseg = 2 * a.nscenes;
    const int64_t total = a.rseg_off[nseg];
    WalkStack<PACK> stk;
    int sp = 0;
    int64_t r = 0;
    int k = 0;
    bool any = false, has = false, exhausted = false, ok = true, fin = false;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
    RayInv ri{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nd = 0.f;
    WalkHit h{0.f, 0.f, 0.f, -1};
    SceneDesc sd{nullptr, nullptr, 0, 0};
    int32_t node = -1, leaf_start = 0, leaf_cnt = 0;
    WorkCount wc;

    auto finish = [&]() {
        if (any) {
            a.occ[r] = h.prim >= 0 ? 1 : 0;
        } else {
            const bool hit = h.prim >= 0;
            a.prim[r] = h.prim;
            a.t[r] = hit ? h.t : 0.f;
            a.b1[r] = hit ? h.b1 : 0.f;
            a.b2[r] = hit ? h.b2 : 0.f;
        }
        if (!ok) atomicAdd(&a.status[kStatusOverflow], 1);
        has = false;
        fin = true;
    };
    auto pop = [&]() -> bool {
        while (sp > 0) {
            --sp;
            int32_t ref, cnt;
            if (stk.get(sp, &ref, &cnt) <= h.t) {
                if (cnt == 0) {
                    node = ref;
                } else {
                    node = -1;
                    leaf_start = ~ref;
                    leaf_cnt = cnt;
                }
                return true;
            }
        }
        return false;
    };

    for (;;) {
        fin = false;
        const unsigned need = __ballot_sync(full, !has && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.head, (unsigned long long)__popc(need));
            base = __shfl_sync(full, base, leader);
            if (!has && !exhausted) {
                const int64_t slot = (int64_t)base + __popc(need & lt);
                if (slot >= total) {
                    exhausted = true;
                } else {
                    int lo = 0, hi = nseg;
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (a.rseg_off[mid] <= slot) lo = mid;
                        else hi = mid;
                    }
                    k = lo >> 1;
                    any = (lo & 1) != 0;
                    r = a.ray_off[lo] + (slot - a.rseg_off[lo]);
                    sd = a.scenes[k];
                    o = any ? a.o4s[r] : a.o4n[r];
                    d = any ? a.d4s[r] : a.d4n[r];
                    nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
                    ri = RayInv{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
                    h = WalkHit{d.w, 0.f, 0.f, -1};
                    sp = 0;
                    node = 0;
                    ok = true;
                    leaf_start = 0;
                    leaf_cnt = sd.unculled;
                    has = true;
                }
            }
        }
        if (!__any_sync(full, has)) {
            if (__all_sync(full, exhausted)) break;
            continue;
        }
        while (has && leaf_cnt == 0) {
            if (node < 0) {
                if (!pop()) {
                    finish();
                    break;
                }
                continue;
            }
            const BvhNode nn = sd.nodes[node];
            float tn0, tn1;
            const bool h0 = slab(ri, nn.n0.x, nn.n0.y, nn.n0.z, nn.n0.w, nn.n2.x, nn.n2.y, o.w, h.t, &tn0);
            const bool h1 = slab(ri, nn.n1.x, nn.n1.y, nn.n1.z, nn.n1.w, nn.n2.z, nn.n2.w, o.w, h.t, &tn1);
            node = -1;
            if (h0 || h1) {
                // any-hit rays take the farther child first (back to front: a
                // shadow ray leaves the surface around its origin; 64-scene
                // step 13.09 -> 12.73 ms)
                const bool near0 = h0 && (!h1 || (any ? tn1 < tn0 : tn0 <= tn1));
                const int32_t cn = near0 ? nn.n3.x : nn.n3.y, kn = near0 ? nn.n3.z : nn.n3.w;
                if (h0 && h1) {
                    const int32_t cf = near0 ? nn.n3.y : nn.n3.x, kf = near0 ? nn.n3.w : nn.n3.z;
                    if (sp < kStackDepth) {
                        stk.put(sp, cf, cf >= 0 ? 0 : kf, near0 ? tn1 : tn0);
                        ++sp;
                    } else {
                        ok = false;
                    }
                }
                if (cn >= 0) {
                    node = cn;
                } else {
                    leaf_start = ~cn;
                    leaf_cnt = kn;
                }
            }
        }
        if (has && leaf_cnt > 0) {
            const bool done = any ? test_run<true, false>(sd.tris, leaf_start, leaf_cnt, o, d, nd, h, wc)
                                  : test_run<false, false>(sd.tris, leaf_start, leaf_cnt, o, d, nd, h, wc);
            leaf_cnt = 0;
            if (done) finish();
        }
        const unsigned m = __match_any_sync(full, fin ? k : -1);
        if (fin && lane == __ffs(m) - 1) atomicMax(&a.done_ns[k], global_ns());
    }
}

// The rays of one query kind of a whole scene set, for the eight-wide walk
// (walks 3 and 4: one launch per kind).  A lane's slot is the ray's index in
// the kind's arrays; its scene is the last one whose first ray is at or
// before it.  A lane keeps only the scene's number and reads the scene's
// pointers from its descriptor when it needs them (L1-resident; keeping
// them in registers made the walk spill: set walk 4 13.26 -> 13.01 ms).
struct SetRays {
    static constexpr bool kSet = true;
    struct Lane {
        int64_t ray;
        int32_t scene;
    };
    const SceneDesc* scenes;
    int32_t nscenes;
    int32_t kind;            // 0 nearest, 1 any-hit
    const int64_t* ray_off;  // [2 * nscenes], segment 2k + kind
    const int64_t* ray_end;
    const float4* o4;
    const float4* d4;
    int32_t* prim;
    float* t;
    float* b1;
    float* b2;
    uint8_t* occ;
    unsigned long long* done_ns;

    __device__ __forceinline__ int64_t count() const { return ray_end[2 * (nscenes - 1) + kind]; }
    __device__ __forceinline__ bool fetch(int64_t slot, Lane& L, float4& o, float4& d) const {
        int lo = 0, hi = nscenes;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (ray_off[2 * mid + kind] <= slot) lo = mid;
            else hi = mid;
        }
        L.ray = slot;
        L.scene = lo;
        o = o4[slot];
        d = d4[slot];
        return true;
    }
    __device__ __forceinline__ const WideNode* nodes(const Lane& L) const { return scenes[L.scene].wide; }
    __device__ __forceinline__ const TriRec* tris(const Lane& L) const { return scenes[L.scene].wtris; }
    __device__ __forceinline__ int32_t unculled(const Lane& L) const { return scenes[L.scene].unculled; }
    template <bool ANY>
    __device__ __forceinline__ void store(const Lane& L, const WalkHit& h) const {
        if (ANY) {
            occ[L.ray] = h.prim >= 0 ? 1 : 0;
        } else {
            const bool hit = h.prim >= 0;
            prim[L.ray] = h.prim;
            t[L.ray] = hit ? h.t : 0.f;
            b1[L.ray] = hit ? h.b1 : 0.f;
            b2[L.ray] = hit ? h.b2 : 0.f;
        }
    }
    __device__ __forceinline__ int scene(const Lane& L) const { return L.scene; }
    __device__ __forceinline__ void stamp(int sc) const { atomicMax(&done_ns[sc], global_ns()); }
};

}  // namespace pbg

using namespace pbg;

struct pbg_sceneset {
    int device = 0;
    int32_t nscenes = 0;
    cudaStream_t capture_stream = nullptr;
    DeviceBuffer nodes, tris, descs, err;
    DeviceBuffer wnodes, wtris;  // every scene's eight-wide tree and record copy
    bool wide_ok = false;        // every scene's tree fits the wide format
    DeviceBuffer head, remaining, done_ns, start_ns;
    std::vector<int64_t> ntri;
    // Segment tables (item_off ++ ray_off ++ ray_end ++ rseg_off) with the
    // graph captured over each: two, so that a caller alternating between
    // two sets of offsets (two halves of the scenes) replays both.
    struct Slot {
        std::vector<int64_t> host;
        DeviceBuffer dev;
        cudaGraphExec_t exec = nullptr;
        std::vector<uintptr_t> key;
        uint64_t used = 0;
    } slot[2];
    int cur = 0;       // the slot of the call in progress
    uint64_t tick = 0;
    pbg_batch_params tuned{};
    int sm_count = 0;
};

namespace {

// walk: 1 = work items of `tile` rays (batch_trace_kernel), 2 = per-lane
// persistent refill (batch_persistent_kernel; tile only sizes the items of
// the completion bookkeeping), 3 / 4 = per-lane persistent refill over the
// eight-wide trees, one launch per query kind (4: the warp's triangle tests
// spread over its lanes); 128 threads.
struct Shape {
    int tile, ctas_per_sm, threads, walk;
};

int max_ctas_per_sm(int threads, int walk) {
    int n = 0;
    const cudaError_t e =
        walk == 3   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &n, wide_walk_kernel<false, false, false, SetRays>, kWideThreads, 0)
        : walk == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &n, wide_walk_kernel<false, false, true, SetRays>, kWideThreads, 0)
        : walk == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_persistent_kernel<true>, threads, 0)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_trace_kernel, threads, 0);
    if (e != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

Shape resolve_shape(const pbg_sceneset* set, const pbg_batch_params* p) {
    Shape s{set->tuned.tile, set->tuned.ctas_per_sm, set->tuned.threads, set->tuned.walk};
    if (p && p->tile > 0) s.tile = p->tile;
    if (p && p->threads > 0) s.threads = p->threads;
    if (p && p->ctas_per_sm > 0) s.ctas_per_sm = p->ctas_per_sm;
    if (p && p->walk > 0) s.walk = p->walk;
    if (s.tile <= 0) s.tile = 64;
    if (s.threads <= 0) s.threads = 128;
    if (s.walk <= 0) s.walk = 1;
    if (s.walk == 3 || s.walk == 4) s.threads = kWideThreads;
    if (s.ctas_per_sm <= 0) s.ctas_per_sm = max_ctas_per_sm(s.threads, s.walk);
    return s;
}

bool shape_ok(const Shape& s) {
    return s.tile >= 32 && s.tile <= 8192 && s.tile % 32 == 0 && s.threads >= 32 &&
           s.threads <= kBatchMaxThreads && s.threads % 32 == 0 && s.ctas_per_sm >= 1 &&
           s.ctas_per_sm <= 64 && s.walk >= 1 && s.walk <= 4;
}

bool offsets_ok(const int64_t* off, int32_t n) {
    if (!off) return false;
    if (off[0] != 0) return false;
    for (int32_t k = 0; k < n; ++k)
        if (off[k + 1] < off[k]) return false;
    return true;
}

// item_off ++ ray_off ++ ray_end ++ rseg_off for this tile.
void make_table(int32_t n, const int64_t* near_off, const int64_t* occ_off, int tile,
                std::vector<int64_t>* out) {
    const int nseg = 2 * n;
    out->assign((size_t)(nseg + 1 + 2 * nseg + nseg + 1), 0);
    int64_t* item = out->data();
    int64_t* roff = item + nseg + 1;
    int64_t* rend = roff + nseg;
    int64_t* rseg = rend + nseg;
    int64_t acc = 0, racc = 0;
    for (int k = 0; k < n; ++k)
        for (int kind = 0; kind < 2; ++kind) {
            const int64_t* off = kind ? occ_off : near_off;
            const int64_t b = off ? off[k] : 0, e = off ? off[k + 1] : 0;
            const int seg = 2 * k + kind;
            item[seg] = acc;
            roff[seg] = b;
            rend[seg] = e;
            rseg[seg] = racc;
            acc += (e - b + tile - 1) / tile;
            racc += e - b;
        }
    item[nseg] = acc;
    rseg[nseg] = racc;
}

struct Call {
    const float *o4n, *d4n;
    const int64_t* near_off;
    int32_t* prim;
    float *t, *b1, *b2;
    const float *o4s, *d4s;
    const int64_t* occ_off;
    uint8_t* occ;
};

BatchArgs make_args(pbg_sceneset* set, const Call& c, int tile) {
    BatchArgs a{};
    a.scenes = (const SceneDesc*)set->descs.ptr;
    a.nscenes = set->nscenes;
    a.tile = tile;
    const int nseg = 2 * set->nscenes;
    const int64_t* table = (const int64_t*)set->slot[set->cur].dev.ptr;
    a.item_off = table;
    a.ray_off = table + nseg + 1;
    a.ray_end = table + nseg + 1 + nseg;
    a.rseg_off = table + nseg + 1 + 2 * nseg;
    a.o4n = (const float4*)c.o4n;
    a.d4n = (const float4*)c.d4n;
    a.prim = c.prim;
    a.t = c.t;
    a.b1 = c.b1;
    a.b2 = c.b2;
    a.o4s = (const float4*)c.o4s;
    a.d4s = (const float4*)c.d4s;
    a.occ = c.occ;
    a.head = (unsigned long long*)set->head.ptr;
    a.remaining = (int32_t*)set->remaining.ptr;
    a.done_ns = (unsigned long long*)set->done_ns.ptr;
    a.start_ns = (unsigned long long*)set->start_ns.ptr;
    a.status = (int*)set->err.ptr;
    return a;
}

int launch_pair(pbg_sceneset* set, const BatchArgs& a, const Shape& s, cudaStream_t st) {
    batch_reset_kernel<<<(unsigned)((set->nscenes + 255) / 256), 256, 0, st>>>(a);
    PBG_CUDA(cudaGetLastError());
    const unsigned grid = (unsigned)(s.ctas_per_sm * set->sm_count);
    if (s.walk == 3 || s.walk == 4) {
        // the nearest-hit rays of every scene, then the any-hit rays
        for (int kind = 0; kind < 2; ++kind) {
            const SetRays src{a.scenes, a.nscenes, kind, a.ray_off, a.ray_end,
                              kind ? a.o4s : a.o4n, kind ? a.d4s : a.d4n, a.prim, a.t, a.b1, a.b2, a.occ,
                              a.done_ns};
            auto kern = kind ? (s.walk == 4 ? wide_walk_kernel<true, false, true, SetRays>
                                            : wide_walk_kernel<true, false, false, SetRays>)
                             : (s.walk == 4 ? wide_walk_kernel<false, false, true, SetRays>
                                            : wide_walk_kernel<false, false, false, SetRays>);
            kern<<<grid, kWideThreads, 0, st>>>(src, a.status, a.head + kind, nullptr);
            PBG_CUDA(cudaGetLastError());
        }
        return PBG_OK;
    }
    if (s.walk == 2) {
        // scene-local record starts below 2^24 fit a packed stack entry
        int64_t max_ntri = 0;
        for (int64_t k : set->ntri) max_ntri = std::max(max_ntri, k);
        if (max_ntri < (1 << 24))
            batch_persistent_kernel<true><<<grid, (unsigned)s.threads, 0, st>>>(a);
        else
            batch_persistent_kernel<false><<<grid, (unsigned)s.threads, 0, st>>>(a);
    } else
        batch_trace_kernel<<<grid, (unsigned)s.threads, 0, st>>>(a);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

// Validates the call, uploads the segment table if it changed.
int prepare(pbg_sceneset* set, const Call& c, const Shape& s, cudaStream_t st, uint64_t* rays) {
    const int32_t n = set->nscenes;
    if (c.near_off && !offsets_ok(c.near_off, n)) {
        set_last_error("pbg_sceneset_trace: near_offsets must start at 0 and not decrease");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (c.occ_off && !offsets_ok(c.occ_off, n)) {
        set_last_error("pbg_sceneset_trace: occ_offsets must start at 0 and not decrease");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    const int64_t nn = c.near_off ? c.near_off[n] : 0, ns = c.occ_off ? c.occ_off[n] : 0;
    if ((nn > 0 && (!c.o4n || !c.d4n || !c.prim || !c.t || !c.b1 || !c.b2)) ||
        (ns > 0 && (!c.o4s || !c.d4s || !c.occ))) {
        set_last_error("pbg_sceneset_trace: NULL ray or result array");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if ((s.walk == 3 || s.walk == 4) && !set->wide_ok) {
        set_last_error("pbg_sceneset_trace: walks 3 and 4 need every scene's tree in the eight-wide format");
        return PBG_ERR_UNSUPPORTED;
    }
    if (!shape_ok(s)) {
        set_last_error("pbg_sceneset_trace: tile and threads must be multiples of 32 (tile <= 8192, "
                       "threads <= 256), ctas_per_sm in [1, 64]");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    std::vector<int64_t> table;
    make_table(n, c.near_off, c.occ_off, s.tile, &table);
    for (int k = 0; k < n; ++k)
        if (table[(size_t)(2 * k + 2)] - table[(size_t)(2 * k)] > (int64_t)INT32_MAX) {
            set_last_error("pbg_sceneset_trace: too many work items in one scene");
            return PBG_ERR_INVALID_ARGUMENT;
        }
    int hit = -1;
    for (int k = 0; k < 2; ++k)
        if (set->slot[k].host == table) hit = k;
    if (hit < 0) {  // upload into the least recently used slot
        hit = set->slot[0].used <= set->slot[1].used ? 0 : 1;
        auto& sl = set->slot[hit];
        if (sl.exec) cudaGraphExecDestroy(sl.exec);
        sl.exec = nullptr;
        sl.key.clear();
        int rc = ensure(sl.dev, table.size() * sizeof(int64_t));
        if (rc) return rc;
        PBG_CUDA(cudaMemcpyAsync(sl.dev.ptr, table.data(), table.size() * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, st));
        // the host vector must outlive the (possibly asynchronous) copy
        PBG_CUDA(cudaStreamSynchronize(st));
        sl.host.swap(table);
    }
    set->cur = hit;
    set->slot[hit].used = ++set->tick;
    *rays = (uint64_t)(nn + ns);
    return PBG_OK;
}

void destroy_graph(pbg_sceneset* set) {
    for (auto& sl : set->slot) {
        if (sl.exec) cudaGraphExecDestroy(sl.exec);
        sl.exec = nullptr;
        sl.key.clear();
    }
}

int run(pbg_sceneset* set, const Call& c, const Shape& s, bool use_graph, cudaStream_t st,
        bool* replayed) {
    const BatchArgs a = make_args(set, c, s.tile);
    *replayed = false;
    if (!use_graph) return launch_pair(set, a, s, st);
    const uintptr_t key_vals[] = {(uintptr_t)c.o4n, (uintptr_t)c.d4n, (uintptr_t)c.prim,
                                  (uintptr_t)c.t,   (uintptr_t)c.b1,  (uintptr_t)c.b2,
                                  (uintptr_t)c.o4s, (uintptr_t)c.d4s, (uintptr_t)c.occ,
                                  (uintptr_t)set->slot[set->cur].dev.ptr, (uintptr_t)s.tile,
                                  (uintptr_t)s.ctas_per_sm, (uintptr_t)s.threads,
                                  (uintptr_t)s.walk};
    std::vector<uintptr_t> key(std::begin(key_vals), std::end(key_vals));
    auto& sl = set->slot[set->cur];
    if (sl.exec && key == sl.key) {
        *replayed = true;
    } else {
        if (sl.exec) cudaGraphExecDestroy(sl.exec);
        sl.exec = nullptr;
        sl.key.clear();
        cudaGraph_t g = nullptr;
        PBG_CUDA(cudaStreamBeginCapture(set->capture_stream, cudaStreamCaptureModeThreadLocal));
        int rc = launch_pair(set, a, s, set->capture_stream);
        cudaError_t e = cudaStreamEndCapture(set->capture_stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&sl.exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            sl.exec = nullptr;
            return cuda_status(e, "cudaGraphInstantiate");
        }
        sl.key = key;
    }
    PBG_CUDA(cudaGraphLaunch(sl.exec, st));
    return PBG_OK;
}

int read_status(pbg_sceneset* set, cudaStream_t st) {
    int h[4] = {0, 0, 0, 0};
    PBG_CUDA(cudaMemcpyAsync(h, set->err.ptr, sizeof(h), cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    if (h[kStatusOverflow] != 0) {
        PBG_CUDA(cudaMemsetAsync(set->err.ptr, 0, sizeof(h), st));
        set_last_error("device status: BVH walk stack overflow");
        return PBG_ERR_INTERNAL;
    }
    return PBG_OK;
}

}  // namespace

extern "C" {

int pbg_sceneset_create(int32_t nscenes, const float* const* tri9, const int64_t* ntri,
                        int32_t device, pbg_sceneset** out) {
    if (!out) {
        set_last_error("pbg_sceneset_create: out is NULL");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (nscenes < 1 || nscenes > kBatchMaxScenes || !tri9 || !ntri) {
        set_last_error("pbg_sceneset_create: need 1..4096 scenes and their triangle arrays");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    for (int32_t k = 0; k < nscenes; ++k)
        if (ntri[k] < 0 || ntri[k] > (int64_t)INT32_MAX / 2 || (ntri[k] > 0 && !tri9[k])) {
            set_last_error("pbg_sceneset_create: bad triangle array");
            return PBG_ERR_INVALID_ARGUMENT;
        }
    if (pbg_device_count() == 0) {
        set_last_error("pbg_sceneset_create: no CUDA device");
        return PBG_ERR_NO_DEVICE;
    }
    pbg_sceneset* set = new (std::nothrow) pbg_sceneset();
    if (!set) return PBG_ERR_OUT_OF_MEMORY;
    set->device = device;
    set->nscenes = nscenes;
    set->ntri.assign(ntri, ntri + nscenes);
    auto fail = [&](int code) {
        pbg_sceneset_destroy(set);
        return code;
    };
    {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) return fail(cuda_status(e, "cudaSetDevice"));
        e = cudaStreamCreateWithFlags(&set->capture_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return fail(cuda_status(e, "cudaStreamCreate"));
        e = cudaDeviceGetAttribute(&set->sm_count, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess) return fail(cuda_status(e, "cudaDeviceGetAttribute"));
    }
    // BVHs on the host cores, one scene per task, each also collapsed to the
    // eight-wide tree (wide records: original triangle of each position)
    std::vector<HostBvh> hb((size_t)nscenes);
    std::vector<std::vector<WideNode>> wn((size_t)nscenes);
    std::vector<std::vector<int32_t>> worder((size_t)nscenes);
    std::atomic<int32_t> wide_fail{0};
    {
        std::atomic<int32_t> next{0};
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const unsigned nt = std::min<unsigned>(hw, (unsigned)nscenes);
        std::vector<std::thread> pool;
        for (unsigned i = 0; i < nt; ++i)
            pool.emplace_back([&] {
                for (int32_t k; (k = next.fetch_add(1)) < nscenes;) {
                    HostBvh& b = hb[(size_t)k];
                    build_bvh(tri9[k], ntri[k], 4, &b);
                    std::vector<int32_t> src;
                    if (b.nodes.empty() ||
                        !collapse_wide(b.nodes, b.unculled, ntri[k], kWideAbsorb, kWideTriCost, &wn[(size_t)k], &src)) {
                        wide_fail.fetch_add(1);
                        continue;
                    }
                    std::vector<int32_t>& wo = worder[(size_t)k];
                    wo.resize(src.size());
                    for (size_t r = 0; r < src.size(); ++r) wo[r] = b.order.empty() ? src[r] : b.order[(size_t)src[r]];
                }
            });
        for (auto& th : pool) th.join();
    }
    set->wide_ok = wide_fail.load() == 0;
    std::vector<int64_t> node_base((size_t)nscenes + 1, 0), tri_base((size_t)nscenes + 1, 0);
    for (int32_t k = 0; k < nscenes; ++k) {
        node_base[(size_t)k + 1] = node_base[(size_t)k] + (int64_t)hb[(size_t)k].nodes.size();
        tri_base[(size_t)k + 1] = tri_base[(size_t)k] + ntri[k];
    }
    const int64_t total_nodes = node_base[(size_t)nscenes], total_tris = tri_base[(size_t)nscenes];
    std::vector<int64_t> wnode_base((size_t)nscenes + 1, 0);
    for (int32_t k = 0; k < nscenes; ++k)
        wnode_base[(size_t)k + 1] = wnode_base[(size_t)k] + (int64_t)wn[(size_t)k].size();
    int rc;
    if ((rc = ensure(set->nodes, (size_t)total_nodes * sizeof(BvhNode))) ||
        (rc = ensure(set->tris, (size_t)std::max<int64_t>(total_tris, 1) * sizeof(TriRec))) ||
        (rc = ensure(set->descs, (size_t)nscenes * sizeof(SceneDesc))) ||
        (rc = ensure(set->err, 4 * sizeof(int))) || (rc = ensure(set->head, 2 * sizeof(uint64_t))) ||
        (rc = ensure(set->start_ns, sizeof(uint64_t))) ||
        (rc = ensure(set->remaining, (size_t)nscenes * sizeof(int32_t))) ||
        (rc = ensure(set->done_ns, (size_t)nscenes * sizeof(uint64_t))))
        return fail(rc);
    if (set->wide_ok &&
        ((rc = ensure(set->wnodes, (size_t)std::max<int64_t>(wnode_base[(size_t)nscenes], 1) * sizeof(WideNode))) ||
         (rc = ensure(set->wtris, (size_t)std::max<int64_t>(total_tris, 1) * sizeof(TriRec)))))
        return fail(rc);
    if (cudaMemset(set->err.ptr, 0, 4 * sizeof(int)) != cudaSuccess)
        return fail(cuda_status(cudaGetLastError(), "cudaMemset"));
    std::vector<SceneDesc> descs((size_t)nscenes);
    int64_t max_ntri = 0;
    for (int32_t k = 0; k < nscenes; ++k) max_ntri = std::max(max_ntri, ntri[k]);
    DeviceBuffer v9, ord;
    if ((rc = ensure(v9, (size_t)std::max<int64_t>(max_ntri, 1) * 9 * sizeof(float))) ||
        (rc = ensure(ord, (size_t)std::max<int64_t>(max_ntri, 1) * sizeof(int32_t)))) {
        release(v9);
        release(ord);
        return fail(rc);
    }
    cudaStream_t st = set->capture_stream;
    for (int32_t k = 0; k < nscenes && rc == PBG_OK; ++k) {
        const HostBvh& b = hb[(size_t)k];
        BvhNode* nodes = (BvhNode*)set->nodes.ptr + node_base[(size_t)k];
        TriRec* tris = (TriRec*)set->tris.ptr + tri_base[(size_t)k];
        WideNode* wide = set->wide_ok ? (WideNode*)set->wnodes.ptr + wnode_base[(size_t)k] : nullptr;
        TriRec* wtris = set->wide_ok ? (TriRec*)set->wtris.ptr + tri_base[(size_t)k] : nullptr;
        descs[(size_t)k] = SceneDesc{nodes, tris, b.unculled, 0, wide, wtris};
        cudaError_t e = cudaMemcpy(nodes, b.nodes.data(), b.nodes.size() * sizeof(BvhNode),
                                   cudaMemcpyHostToDevice);
        if (e == cudaSuccess && wide && !wn[(size_t)k].empty())
            e = cudaMemcpy(wide, wn[(size_t)k].data(), wn[(size_t)k].size() * sizeof(WideNode),
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess && ntri[k] > 0) {
            e = cudaMemcpy(v9.ptr, tri9[k], (size_t)ntri[k] * 9 * sizeof(float), cudaMemcpyHostToDevice);
            if (e == cudaSuccess)
                e = cudaMemcpy(ord.ptr, b.order.data(), (size_t)ntri[k] * sizeof(int32_t),
                               cudaMemcpyHostToDevice);
            if (e == cudaSuccess) {
                rc = launch_build_tris((const float*)v9.ptr, (const int32_t*)ord.ptr, ntri[k], tris, st);
                if (rc == PBG_OK) e = cudaStreamSynchronize(st);
            }
            if (e == cudaSuccess && rc == PBG_OK && wtris) {  // the wide tree's record order
                e = cudaMemcpy(ord.ptr, worder[(size_t)k].data(), (size_t)ntri[k] * sizeof(int32_t),
                               cudaMemcpyHostToDevice);
                if (e == cudaSuccess) {
                    rc = launch_build_tris((const float*)v9.ptr, (const int32_t*)ord.ptr, ntri[k], wtris, st);
                    if (rc == PBG_OK) e = cudaStreamSynchronize(st);
                }
            }
        }
        if (e != cudaSuccess && rc == PBG_OK) rc = cuda_status(e, "pbg_sceneset_create upload");
    }
    release(v9);
    release(ord);
    if (rc) return fail(rc);
    if (cudaMemcpy(set->descs.ptr, descs.data(), descs.size() * sizeof(SceneDesc),
                   cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(cuda_status(cudaGetLastError(), "cudaMemcpy(descs)"));
    set->tuned.use_graph = 1;
    *out = set;
    return PBG_OK;
}

void pbg_sceneset_destroy(pbg_sceneset* set) {
    if (!set) return;
    cudaSetDevice(set->device);
    cudaDeviceSynchronize();
    destroy_graph(set);
    DeviceBuffer* all[] = {&set->nodes,       &set->tris, &set->descs,     &set->err,     &set->slot[0].dev,
                           &set->slot[1].dev, &set->head, &set->remaining, &set->done_ns, &set->start_ns,
                           &set->wnodes,      &set->wtris};
    for (DeviceBuffer* b : all) release(*b);
    if (set->capture_stream) cudaStreamDestroy(set->capture_stream);
    delete set;
}

int pbg_sceneset_trace(pbg_sceneset* set, const float* o4n, const float* d4n,
                       const int64_t* near_offsets, int32_t* prim, float* t, float* b1, float* b2,
                       const float* o4s, const float* d4s, const int64_t* occ_offsets, uint8_t* occ,
                       const pbg_batch_params* params, pbg_batch_stats* stats, double* scene_ms,
                       void* stream) {
    if (!set) {
        set_last_error("pbg_sceneset_trace: set is NULL");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(set->device);
    cudaStream_t st = (cudaStream_t)stream;
    const Call c{o4n, d4n, near_offsets, prim, t, b1, b2, o4s, d4s, occ_offsets, occ};
    const Shape s = resolve_shape(set, params);
    uint64_t rays = 0;
    int rc = prepare(set, c, s, st, &rays);
    if (rc) return rc;
    const bool use_graph = params ? params->use_graph != 0 : set->tuned.use_graph != 0;
    const bool timed = stats || scene_ms;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (timed) {
        PBG_CUDA(cudaEventCreate(&e0));
        PBG_CUDA(cudaEventCreate(&e1));
        PBG_CUDA(cudaEventRecord(e0, st));
    }
    bool replayed = false;
    rc = run(set, c, s, use_graph, st, &replayed);
    if (rc == PBG_OK && timed) {
        cudaEventRecord(e1, st);
        rc = read_status(set, st);
    }
    if (rc == PBG_OK && timed) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const int32_t n = set->nscenes;
        std::vector<unsigned long long> done((size_t)n);
        unsigned long long t0 = 0;
        cudaError_t e = cudaMemcpy(done.data(), set->done_ns.ptr, (size_t)n * sizeof(uint64_t),
                                   cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(&t0, set->start_ns.ptr, sizeof(uint64_t), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_status(e, "pbg_sceneset_trace readback");
        std::vector<double> busy;
        for (int32_t k = 0; k < n && rc == PBG_OK; ++k) {
            const std::vector<int64_t>& ht = set->slot[set->cur].host;
            const bool work = ht[(size_t)(2 * k + 2)] > ht[(size_t)(2 * k)];
            const double v = work && done[(size_t)k] >= t0 ? (double)(done[(size_t)k] - t0) * 1e-6 : 0.0;
            if (scene_ms) scene_ms[k] = v;
            if (work) busy.push_back(v);
        }
        if (stats && rc == PBG_OK) {
            std::sort(busy.begin(), busy.end());
            auto pct = [&](double q) {
                if (busy.empty()) return 0.0;
                size_t i = (size_t)std::ceil(q * (double)busy.size()) - 1;
                return busy[std::min(i, busy.size() - 1)];
            };
            stats->ms = ms;
            stats->scene_ms_p50 = pct(0.50);
            stats->scene_ms_p99 = pct(0.99);
            stats->rays = rays;
            stats->tile = s.tile;
            stats->ctas_per_sm = s.ctas_per_sm;
            stats->threads = s.threads;
            stats->graph_replayed = replayed ? 1 : 0;
            stats->walk = s.walk;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}

int pbg_sceneset_autotune(pbg_sceneset* set, const float* o4n, const float* d4n,
                          const int64_t* near_offsets, int32_t* prim, float* t, float* b1,
                          float* b2, const float* o4s, const float* d4s, const int64_t* occ_offsets,
                          uint8_t* occ, pbg_batch_params* best, void* stream) {
    if (!set) {
        set_last_error("pbg_sceneset_autotune: set is NULL");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(set->device);
    cudaStream_t st = (cudaStream_t)stream;
    const Call c{o4n, d4n, near_offsets, prim, t, b1, b2, o4s, d4s, occ_offsets, occ};
    const int tiles[] = {32, 64, 128, 256};
    const int threads[] = {64, 128, 256};
    cudaEvent_t e0, e1;
    PBG_CUDA(cudaEventCreate(&e0));
    PBG_CUDA(cudaEventCreate(&e1));
    float best_ms = INFINITY;
    Shape win{64, 0, 128, 1};
    int rc = PBG_OK;
    for (int walk = 1; walk <= 4; ++walk)
    for (int th : threads) {
        if (walk >= 3 && (th != kWideThreads || !set->wide_ok)) continue;  // the wide walks run 128 threads
        const int full = max_ctas_per_sm(th, walk);
        const int ctas[] = {full, std::max(1, full / 2)};
        for (int ci = 0; ci < 2 && rc == PBG_OK; ++ci) {
            if (ci == 1 && ctas[1] == ctas[0]) continue;
            for (int tile : tiles) {
                if (walk >= 2 && tile != 64) continue;  // the persistent walks do not use tiles
                const Shape s{tile, ctas[ci], th, walk};
                uint64_t rays = 0;
                if ((rc = prepare(set, c, s, st, &rays))) break;
                bool rep = false;
                if ((rc = run(set, c, s, false, st, &rep))) break;  // warm-up
                cudaEventRecord(e0, st);
                for (int r = 0; r < 2 && rc == PBG_OK; ++r) rc = run(set, c, s, false, st, &rep);
                cudaEventRecord(e1, st);
                if (rc) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    rc = cuda_status(cudaGetLastError(), "autotune");
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best_ms) {
                    best_ms = ms;
                    win = s;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == PBG_OK) rc = read_status(set, st);
    if (rc) return rc;
    set->tuned.tile = win.tile;
    set->tuned.ctas_per_sm = win.ctas_per_sm;
    set->tuned.threads = win.threads;
    set->tuned.walk = win.walk;
    set->tuned.use_graph = 1;
    if (best) *best = set->tuned;
    return PBG_OK;
}

}  // extern "C"
