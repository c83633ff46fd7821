// pbg_bvh.cu -- Accelerator "ray-bvh": rays against a SAH BVH over triangles.
//
// Replaces the fork's co-traversal kernels (bin/cl/intersection6DB_BVH.cl,
// intersection6DB_BVH2.cl, intersectionP6DB_BVH.cl: one thread per top-level
// BVH node walking the ray quadtree and the BVH subtree with a global-memory
// stack, accelerators/rayBVH.cpp:615-1323).  Here one thread owns one ray and
// walks the whole tree with a private stack (pbg_walk.cuh), nearest child
// first.  Rays run in the caller's order (camera and shadow batches from the
// breadth-first renderer are already coherent) or, when the scene asks for
// it, in the 6-D Morton order of the per-batch ray hierarchy
// (pbg_rayorder.cu).  With the learned ordering on (pbg_learn.cu), or with
// cluster hints from the caller, each ray first walks the predicted cluster
// of the BVH's top cut; an any-hit ray whose guess holds an occluder stops
// there.
#include <algorithm>

#include "pbg_internal.h"
#include "pbg_learn.h"
#include "pbg_tma.cuh"
#include "pbg_walk.cuh"

namespace pbg {

constexpr int kBvhThreads = 128;
constexpr int kBvhMinBlocks = 4;  // CTAs per SM: measured best of 4, 5, 6, 8, 12, 16

template <bool ANY, bool STATS, bool ORDERED>
__global__ void __launch_bounds__(kBvhThreads, kBvhMinBlocks)
    bvh_kernel(const BvhNode* __restrict__ nodes, const TriRec* __restrict__ tris, int32_t unculled,
               const float4* __restrict__ ro, const float4* __restrict__ rd,
               const uint8_t* __restrict__ valid, const int32_t* __restrict__ perm, int64_t n,
               int32_t* __restrict__ prim_out, float* __restrict__ t_out,
               float* __restrict__ b1_out, float* __restrict__ b2_out, uint8_t* __restrict__ occ,
               int* status, unsigned long long* wcount, const uint16_t* __restrict__ pred,
               const int32_t* __restrict__ cref) {
    const int64_t slot = (int64_t)blockIdx.x * kBvhThreads + threadIdx.x;
    if (slot >= n) return;
    const int64_t ray = perm ? (int64_t)perm[slot] : slot;
    const bool active = valid == nullptr || valid[ray] != 0;
    if (!active) {
        if (ANY) {
            occ[ray] = 0;
            if (prim_out) prim_out[ray] = -1;
        } else {
            prim_out[ray] = -1;
            t_out[ray] = 0.f;
            b1_out[ray] = 0.f;
            b2_out[ray] = 0.f;
        }
        return;
    }
    WorkCount wc;
    const float4 o = ro[ray], d = rd[ray];
    WalkHit h{d.w, 0.f, 0.f, -1};
    int32_t fref = INT32_MIN, fcnt = 0;
    if (ORDERED) {
        const int c = pred[ray];
        if (c < kClusters) {  // anything else (kNoCluster included): no hint
            fref = cref[2 * c];
            fcnt = cref[2 * c + 1];
        }
    }
    const bool ok = bvh_walk<ANY, STATS, ORDERED>(nodes, tris, unculled, o, d, fref, fcnt, h, wc);
    if (!ok) atomicAdd(&status[kStatusOverflow], 1);
    if (STATS) wc.flush(wcount);
    if (ANY) {
        occ[ray] = h.prim >= 0 ? 1 : 0;
        if (prim_out) prim_out[ray] = h.prim;  // the occluder found (labels, hints)
        return;
    }
    prim_out[ray] = h.prim;
    t_out[ray] = h.prim >= 0 ? h.t : 0.f;
    b1_out[ray] = h.prim >= 0 ? h.b1 : 0.f;
    b2_out[ray] = h.prim >= 0 ? h.b2 : 0.f;
}

// Co-traversal of the ray hierarchy with the BVH (walk = 3): the batch is
// put in the ray hierarchy's leaf order (6-D Morton keys of origin and
// direction, or the declared ray image's Morton order; walk = 4 keeps the
// caller's order, already coherent for image-ordered batches), and each warp takes
// one leaf of 32 rays and walks the BVH with them as one packet: a node is
// visited when any of the warp's rays hits it, every lane tests its own ray
// against both children's boxes, leaves are tested by the lanes whose rays
// reach them, and the stack is the warp's, in shared memory.  The nearer
// child by the lanes' majority vote goes first.  The replaced reference
// kernels pair ray-hierarchy nodes with BVH nodes level by level
// (rayBVH.cpp:615-836, intersection6DB_BVH.cl); the warp packet makes the
// same pairing one leaf at a time.  Warps take leaves from a global counter.
constexpr int kPacketThreads = 128;
constexpr int kPacketStack = 64;

template <bool ANY, bool STATS>
__global__ void __launch_bounds__(kPacketThreads)
    bvh_packet_kernel(const BvhNode* __restrict__ nodes, const TriRec* __restrict__ tris, int32_t unculled,
                      const float4* __restrict__ ro, const float4* __restrict__ rd,
                      const uint8_t* __restrict__ valid, const int32_t* __restrict__ perm, int64_t n,
                      int32_t* __restrict__ prim_out, float* __restrict__ t_out, float* __restrict__ b1_out,
                      float* __restrict__ b2_out, uint8_t* __restrict__ occ, int* status,
                      unsigned long long* next, unsigned long long* wcount) {
    __shared__ int32_t stk[kPacketThreads / 32][kPacketStack];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const int64_t npk = (n + 31) / 32;
    WorkCount wc;
    bool overflow = false;
    for (;;) {
        unsigned long long pk = 0;
        if (lane == 0) pk = atomicAdd(next, 1ull);
        pk = __shfl_sync(full, pk, 0);
        if ((int64_t)pk >= npk) break;
        const int64_t slot = (int64_t)pk * 32 + lane;
        const int64_t ray = slot < n ? (perm ? (int64_t)perm[slot] : slot) : -1;
        const bool active = ray >= 0 && (valid == nullptr || valid[ray] != 0);
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = make_float4(0.f, 0.f, 1.f, 0.f);
        if (active) {
            o = ro[ray];
            d = rd[ray];
        }
        const float ndd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
        const RayInv ri{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
        WalkHit h{d.w, 0.f, 0.f, -1};
        bool done = !active;
        if (!done && unculled > 0) done = test_run<ANY, STATS>(tris, 0, unculled, o, d, ndd, h, wc);
        int sp = 0;  // warp-uniform
        int32_t node = 0;
        for (;;) {
            if (__all_sync(full, done)) break;
            const BvhNode nd_ = nodes[node];
            float tn0 = 0.f, tn1 = 0.f;
            bool h0 = false, h1 = false;
            if (!done) {
                if (STATS) wc.node += 2;
                h0 = slab(ri, nd_.n0.x, nd_.n0.y, nd_.n0.z, nd_.n0.w, nd_.n2.x, nd_.n2.y, o.w, h.t, &tn0);
                h1 = slab(ri, nd_.n1.x, nd_.n1.y, nd_.n1.z, nd_.n1.w, nd_.n2.z, nd_.n2.w, o.w, h.t, &tn1);
            }
            const int32_t c0 = nd_.n3.x, c1 = nd_.n3.y;
            const unsigned both = __ballot_sync(full, h0 && h1);
            // any-hit packets vote for the farther child (terrain shadow batches 0.551 -> 0.547 ms)
            const unsigned near1 = __ballot_sync(full, h0 && h1 && (ANY ? tn0 < tn1 : tn1 < tn0));
            const bool first1 = 2 * __popc(near1) > __popc(both);
            // leaf children at once, the nearer one first
            for (int q = 0; q < 2; ++q) {
                const int side = first1 ? 1 - q : q;
                const int32_t c = side ? c1 : c0;
                const bool hh = side ? h1 : h0;
                if (c < 0 && __any_sync(full, hh && !done)) {
                    if (hh && !done) {
                        if (STATS) wc.leaf++;
                        done = test_run<ANY, STATS>(tris, ~c, side ? nd_.n3.w : nd_.n3.z, o, d, ndd, h, wc);
                    }
                }
            }
            const bool g0 = c0 >= 0 && __any_sync(full, h0 && !done);
            const bool g1 = c1 >= 0 && __any_sync(full, h1 && !done);
            if (g0 && g1) {
                const int32_t nearc = first1 ? c1 : c0, farc = first1 ? c0 : c1;
                if (sp < kPacketStack) {
                    if (lane == 0) stk[warp][sp] = farc;
                    ++sp;
                } else {
                    overflow = true;
                }
                node = nearc;
            } else if (g0 || g1) {
                node = g0 ? c0 : c1;
            } else {
                if (sp == 0) break;
                __syncwarp();
                node = stk[warp][--sp];
                __syncwarp();
            }
        }
        if (ray < 0) continue;
        if (ANY) {
            occ[ray] = h.prim >= 0 ? 1 : 0;
            if (prim_out) prim_out[ray] = h.prim;
        } else {
            prim_out[ray] = h.prim;
            t_out[ray] = h.prim >= 0 ? h.t : 0.f;
            b1_out[ray] = h.prim >= 0 ? h.b1 : 0.f;
            b2_out[ray] = h.prim >= 0 ? h.b2 : 0.f;
        }
    }
    if (overflow && lane == 0) atomicAdd(&status[kStatusOverflow], 1);
    if (STATS) wc.flush(wcount);
}

// Persistent "while-while" form for incoherent batches (one thread per ray
// leaves most lanes of a warp idle: rays finish at different times and leaf
// tests run for a few lanes at a time).  Each lane takes a new ray from a
// global counter as soon as its ray is done, so warps stay full; and each
// outer iteration first walks inner nodes until the lane holds a leaf (or
// its ray ends), then runs the leaf tests, so the warp tests leaves
// together.  The stack keeps leaf children with their triangle counts.
// Same culling, order-independent merge and results as bvh_kernel.
constexpr int kPersistThreads = 128;
constexpr int kPersistMinBlocks = 10;  // CTAs per SM: measured best of 6, 8, 9, 10, 12, 16

// ORDERED: the learned ordering's predicted cluster (pred, cref as in
// bvh_kernel) is walked first, then the whole tree skipping it.  STATS: the
// counting variant (profiling level 2) tallies node tests, leaves and
// triangle tests into wcount.
template <bool ANY, bool ORDERED, bool STATS, bool PACK>
__global__ void __launch_bounds__(kPersistThreads, kPersistMinBlocks)
    bvh_persistent_kernel(const BvhNode* __restrict__ nodes, const TriRec* __restrict__ tris,
                          int32_t unculled, const float4* __restrict__ ro, const float4* __restrict__ rd,
                          const uint8_t* __restrict__ valid, const int32_t* __restrict__ perm, int64_t n,
                          int32_t* __restrict__ prim_out, float* __restrict__ t_out,
                          float* __restrict__ b1_out, float* __restrict__ b2_out,
                          uint8_t* __restrict__ occ, int* status, unsigned long long* next,
                          const uint16_t* __restrict__ pred, const int32_t* __restrict__ cref,
                          unsigned long long* wcount) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    WalkStack<PACK> stk;
    int sp = 0;
    int64_t ray = 0;
    bool has = false, exhausted = false, ok = true;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
    RayInv ri{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nd = 0.f;
    WalkHit h{0.f, 0.f, 0.f, -1};
    int32_t node = -1, leaf_start = 0, leaf_cnt = 0, skip = INT32_MIN;
    int32_t leafb_start = 0, leafb_cnt = 0;  // a second, postponed leaf
    float leafb_t = 0.f;
    int32_t leafc_start = 0, leafc_cnt = 0;  // a third
    float leafc_t = 0.f;
    WorkCount wc;

    auto finish = [&]() {
        if (ANY) {
            occ[ray] = h.prim >= 0 ? 1 : 0;
            if (prim_out) prim_out[ray] = h.prim;
        } else {
            const bool hit = h.prim >= 0;
            prim_out[ray] = h.prim;
            t_out[ray] = hit ? h.t : 0.f;
            b1_out[ray] = hit ? h.b1 : 0.f;
            b2_out[ray] = hit ? h.b2 : 0.f;
        }
        if (!ok) atomicAdd(&status[kStatusOverflow], 1);
        has = false;
    };
    // a leaf reached by the walk: the first pending slot, else the second
    auto take_leaf = [&](int32_t start, int32_t cnt, float tnear) {
        if (leaf_cnt == 0) {
            leaf_start = start;
            leaf_cnt = cnt;
        } else {
            if (leafb_cnt == 0) {
                leafb_start = start;
                leafb_cnt = cnt;
                leafb_t = tnear;
            } else {
                leafc_start = start;
                leafc_cnt = cnt;
                leafc_t = tnear;
            }
        }
    };
    // next stack entry that can still hold a hit; false when the stack is empty
    auto pop = [&]() -> bool {
        while (sp > 0) {
            --sp;
            int32_t ref, cnt;
            const float te = stk.get(sp, &ref, &cnt);
            if (te <= h.t) {
                if (cnt == 0) {
                    node = ref;
                } else {
                    node = -1;
                    take_leaf(~ref, cnt, te);
                }
                return true;
            }
        }
        return false;
    };

    for (;;) {
        // refill the lanes whose ray is done
        const unsigned need = __ballot_sync(full, !has && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(need));
            base = __shfl_sync(full, base, leader);
            if (!has && !exhausted) {
                const int64_t slot = (int64_t)base + __popc(need & lt);
                if (slot >= n) {
                    exhausted = true;
                } else {
                    ray = perm ? (int64_t)perm[slot] : slot;
                    if (valid != nullptr && valid[ray] == 0) {
                        h = WalkHit{0.f, 0.f, 0.f, -1};
                        ok = true;
                        finish();  // invalid: a miss, no walk
                    } else {
                        o = ro[ray];
                        d = rd[ray];
                        nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
                        ri = RayInv{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
                        h = WalkHit{d.w, 0.f, 0.f, -1};
                        sp = 0;
                        node = 0;
                        ok = true;
                        leaf_start = 0;
                        leaf_cnt = unculled;  // degenerate records first
                        leafb_cnt = 0;
                        leafc_cnt = 0;
                        has = true;
                        skip = INT32_MIN;
                        if (ORDERED) {
                            const int c = pred[ray];
                            if (c < kClusters) {
                                // the root after the predicted cluster
                                skip = cref[2 * c];
                                stk.put(0, 0, 0, -INFINITY);
                                sp = 1;
                                if (skip >= 0) {
                                    node = skip;
                                } else {
                                    stk.put(1, skip, cref[2 * c + 1], -INFINITY);
                                    sp = 2;
                                    node = -1;
                                }
                            }
                        }
                    }
                }
            }
        }
        if (!__any_sync(full, has)) {
            if (__all_sync(full, exhausted)) break;
            continue;
        }
        // Inner nodes until every lane holds a leaf or has ended its ray; a
        // lane that already holds one keeps walking for up to two more while
        // others still search, so the leaf tests below run with fuller warps
        // (two postponed leaves: 1,202 -> 1,205 Mrays/s on the path frame).
        for (;;) {
            const bool searching = has && leaf_cnt == 0;
            if (!__any_sync(full, searching)) break;
            if (!has || leafc_cnt > 0) continue;
            if (node < 0) {
                if (!pop() && leaf_cnt == 0) finish();  // stack empty, nothing pending: done
                continue;
            }
            const BvhNode nn = nodes[node];
            if (STATS) wc.node += 2;
            float tn0, tn1;
            bool h0 = slab(ri, nn.n0.x, nn.n0.y, nn.n0.z, nn.n0.w, nn.n2.x, nn.n2.y, o.w, h.t, &tn0);
            bool h1 = slab(ri, nn.n1.x, nn.n1.y, nn.n1.z, nn.n1.w, nn.n2.z, nn.n2.w, o.w, h.t, &tn1);
            if (ORDERED) {  // the predicted cluster has been walked already
                h0 = h0 && nn.n3.x != skip;
                h1 = h1 && nn.n3.y != skip;
            }
            node = -1;
            if (h0 || h1) {
                const bool near0 = h0 && (!h1 || tn0 <= tn1);
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
                    take_leaf(~cn, kn, near0 ? tn0 : tn1);
                }
            }
        }
        // the leaf tests, converged
        if (has && leaf_cnt > 0) {
            if (STATS) wc.leaf++;
            bool done = test_run<ANY, STATS>(tris, leaf_start, leaf_cnt, o, d, nd, h, wc);
            leaf_cnt = 0;
            if (!done && leafb_cnt > 0 && leafb_t <= h.t) {
                if (STATS) wc.leaf++;
                done = test_run<ANY, STATS>(tris, leafb_start, leafb_cnt, o, d, nd, h, wc);
            }
            leafb_cnt = 0;
            if (!done && leafc_cnt > 0 && leafc_t <= h.t) {
                if (STATS) wc.leaf++;
                done = test_run<ANY, STATS>(tris, leafc_start, leafc_cnt, o, d, nd, h, wc);
            }
            leafc_cnt = 0;
            if (done) finish();
        }
    }
    if (STATS) wc.flush(wcount);
}

int ray_order(pbg_scene* s, const float4* o, const float4* d, int64_t n, const int32_t** perm,
              cudaStream_t st);

// cluster_hint: a caller's cluster per ray (kNoCluster or any value outside
// 0..kClusters-1 = none), walked first; else
// the learned ordering's prediction when it is on for this kind of query.
// occluders (any-hit): receives the triangle each walk found, or -1.
template <bool ANY>
static int bvh_launch(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid,
                      int64_t n, int32_t* prim, float* t, float* b1, float* b2, uint8_t* occ,
                      const uint16_t* cluster_hint, int32_t* occluders, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    const int32_t* perm = nullptr;
    if (s->params.ray_sort > 0) {
        int rc = ray_order(s, o, d, n, &perm, st);
        if (rc) return rc;
    }
    const uint16_t* pred = nullptr;
    const int32_t* cref = nullptr;
    Learner* lrn = s->learn;
    const bool learning = lrn && lrn->enabled && (lrn->queries & (ANY ? 2 : 1));
    int rc = PBG_OK;
    if (cluster_hint) {
        if ((rc = ensure_clusters(s))) return rc;
        pred = cluster_hint;
        cref = (const int32_t*)s->learn->cluster_ref.ptr;
    } else if (learning) {
        rc = learn_predict(s, o, d, n, &pred, &cref, st);
    }
    if (rc) return rc;
    // any-hit batches of a learning scene record their occluders as labels
    if (ANY && learning && !occluders) {
        if ((rc = ensure(lrn->occ_prim, (size_t)n * sizeof(int32_t)))) return rc;
        occluders = (int32_t*)lrn->occ_prim.ptr;
    }
    if (ANY) prim = occluders;
    const unsigned grid = (unsigned)((n + kBvhThreads - 1) / kBvhThreads);
    const BvhNode* nodes = (const BvhNode*)s->bvh.ptr;
    const TriRec* tris = (const TriRec*)s->tris.ptr;
    int* status = (int*)s->err.ptr;
    unsigned long long* wc = (unsigned long long*)s->workc.ptr;
    // bounce batches are incoherent: the reference's bounce form of Intersect
    // is the one with a validity mask (rayhierarchy.cpp:602-813)
    const int hint = s->walk_hint >= 0 ? s->walk_hint : (!ANY && valid != nullptr ? 1 : 0);
    const int tuned = s->tune.bvh_walk[ANY ? 1 : 0][hint == 1 ? 1 : 0];
    // untuned: the walks the autotuner picked on both benchmark scenes' batch
    // classes (camera rays 4; their shadow rays 5; bounce rays and their
    // shadows 6), none of them more than 25 % off the class's best there
    const int fallback = hint == 1 ? 6 : (ANY ? 5 : 4);
    int walk = s->params.walk != 0 ? s->params.walk : (tuned != 0 ? tuned : fallback);
    // Host-buffer calls run the packets in the caller's order: there the
    // batch arrives in parts whose copies overlap the traversal, and sorting
    // each part cost more than its packets gained (terrain frame end to end:
    // 1,888 Mrays/s sorted, 2,639 in the caller's order).
    if (walk == 3 && s->host_call && s->params.walk == 0) walk = 4;
    // the packet walk has no ordered form: with cluster hints or the learned
    // ordering it gives way to the persistent walk
    // walk 3: packets over the ray hierarchy's leaves (the batch sorted into
    // its leaf order); walk 4: packets over the batch in the caller's order
    // (camera rays in image order and the shadow rays that follow them are
    // already coherent)
    const bool packet = (walk == 3 || walk == 4) && !pred;
    // walks 5 and 6: the eight-wide tree (built on first use; a tree that
    // does not fit its format keeps the persistent two-wide walk, as do
    // ordered walks); walk 6 spreads a warp's triangle tests over its lanes
    bool wide = (walk == 5 || walk == 6) && !pred;
    if (wide) {
        bool avail = false;
        if ((rc = ensure_wide(s, &avail, st))) return rc;
        wide = avail;
    }
    const bool persistent = walk == 2 || (walk >= 3 && walk <= 6 && (pred || !(walk == 3 || walk == 4 || wide)));
    const int32_t* order = perm;  // packet walk 3: the ray hierarchy's leaf order (timed as the sort stage)
    if (packet && walk == 3 && !order) {
        int rc3 = ray_order(s, o, d, n, &order, st);
        if (rc3) return rc3;
    }
    prof_begin(s, st);
    if (packet) {
        int rc3 = PBG_OK;
        Work& w = s->work;
        if ((rc3 = ensure(w.counters, 64))) return rc3;
        unsigned long long* next = (unsigned long long*)w.counters.ptr;
        PBG_CUDA(cudaMemsetAsync(next, 0, sizeof(unsigned long long), st));
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bvh_packet_kernel<ANY, false>, kPacketThreads, 0);
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
        int64_t blocks = (int64_t)std::max(per_sm, 1) * sms;
        blocks = std::min<int64_t>(blocks, (n + kPacketThreads - 1) / kPacketThreads);
        const bool stats = s->prof.level >= 2;
        auto kern = stats ? bvh_packet_kernel<ANY, true> : bvh_packet_kernel<ANY, false>;
        kern<<<(unsigned)blocks, kPacketThreads, 0, st>>>(nodes, tris, s->unculled, o, d, valid, order, n, prim, t,
                                                          b1, b2, occ, status, next, stats ? wc : nullptr);
    } else if (wide) {
        rc = ANY ? wide_occluded(s, walk == 6, o, d, valid, perm, n, prim, occ, st)
                 : wide_nearest(s, walk == 6, o, d, valid, perm, n, prim, t, b1, b2, st);
        if (rc) return rc;
    } else if (persistent) {
        // persistent while-while walk: one counter word, zeroed per launch
        Work& w = s->work;
        int rc2 = ensure(w.counters, 64);
        if (rc2) return rc2;
        unsigned long long* next = (unsigned long long*)w.counters.ptr;
        PBG_CUDA(cudaMemsetAsync(next, 0, sizeof(unsigned long long), st));
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bvh_persistent_kernel<ANY, false, false, true>,
                                                      kPersistThreads, 0);
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
        int64_t blocks = (int64_t)std::max(per_sm, 1) * sms;
        blocks = std::min<int64_t>(blocks, (n + kPersistThreads - 1) / kPersistThreads);
        const bool stats = s->prof.level >= 2;
        // packed stack entries: record starts below 2^24, leaves below 128 triangles
        const bool pack = s->ntri < (1 << 24) && (s->params.max_bvh_prim > 0 ? s->params.max_bvh_prim : 4) < 128;
        auto kern = pack ? (pred ? (stats ? bvh_persistent_kernel<ANY, true, true, true>
                                          : bvh_persistent_kernel<ANY, true, false, true>)
                                 : (stats ? bvh_persistent_kernel<ANY, false, true, true>
                                          : bvh_persistent_kernel<ANY, false, false, true>))
                         : (pred ? (stats ? bvh_persistent_kernel<ANY, true, true, false>
                                          : bvh_persistent_kernel<ANY, true, false, false>)
                                 : (stats ? bvh_persistent_kernel<ANY, false, true, false>
                                          : bvh_persistent_kernel<ANY, false, false, false>));
        kern<<<(unsigned)blocks, kPersistThreads, 0, st>>>(nodes, tris, s->unculled, o, d, valid, perm, n,
                                                           prim, t, b1, b2, occ, status, next, pred, cref,
                                                           stats ? wc : nullptr);
    } else if (pred) {
        if (s->prof.level >= 2)
            bvh_kernel<ANY, true, true><<<grid, kBvhThreads, 0, st>>>(
                nodes, tris, s->unculled, o, d, valid, perm, n, prim, t, b1, b2, occ, status, wc, pred, cref);
        else
            bvh_kernel<ANY, false, true><<<grid, kBvhThreads, 0, st>>>(
                nodes, tris, s->unculled, o, d, valid, perm, n, prim, t, b1, b2, occ, status, nullptr, pred,
                cref);
    } else {
        if (s->prof.level >= 2)
            bvh_kernel<ANY, true, false><<<grid, kBvhThreads, 0, st>>>(
                nodes, tris, s->unculled, o, d, valid, perm, n, prim, t, b1, b2, occ, status, wc, nullptr,
                nullptr);
        else
            bvh_kernel<ANY, false, false><<<grid, kBvhThreads, 0, st>>>(
                nodes, tris, s->unculled, o, d, valid, perm, n, prim, t, b1, b2, occ, status, nullptr,
                nullptr, nullptr);
    }
    prof_end(s, st, kStageTraverse, 1);
    PBG_CUDA(cudaGetLastError());
    // records for the learned ordering: first hits, occluders
    if (learning) return learn_collect(s, o, d, prim, n, st);
    return PBG_OK;
}

int bvh_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    return bvh_launch<false>(s, o, d, valid, n, prim, t, b1, b2, nullptr, nullptr, nullptr, st);
}

int bvh_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                 uint8_t* occ, cudaStream_t st) {
    return bvh_launch<true>(s, o, d, valid, n, nullptr, nullptr, nullptr, nullptr, occ, nullptr, nullptr, st);
}

int bvh_nearest_hinted(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                       const uint16_t* hint, int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    return bvh_launch<false>(s, o, d, valid, n, prim, t, b1, b2, nullptr, hint, nullptr, st);
}

int bvh_occluded_hinted(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                        const uint16_t* hint, uint8_t* occ, int32_t* occluders, cudaStream_t st) {
    return bvh_launch<true>(s, o, d, valid, n, nullptr, nullptr, nullptr, nullptr, occ, hint, occluders, st);
}

}  // namespace pbg
