// pbg_wide.cuh -- the walk over an eight-wide BVH (ray-bvh walks 5 and 6,
// and the scene set's wide walks), templated on where its rays come from.
//
// Src supplies: count() rays; fetch(slot, lane, o, d) -> false for a ray
// that is not traced (a miss); nodes / tris / unculled of a lane's scene;
// store<ANY>(lane, hit); kSet with scene(lane) and stamp(scene) for a scene
// set's completion stamps.  The node layout and the walk are described in
// pbg_wide.cu.
#pragma once
#include <vector>

#include "pbg_internal.h"
#ifdef __CUDACC__
#include "pbg_tma.cuh"
#include "pbg_walk.cuh"
#endif

namespace pbg {

struct __align__(16) WideNode {
    float4 plane[12];  // per axis: lo[0-3], lo[4-7], hi[0-3], hi[4-7]
    int4 refs;         // child_base | imask << 24, tri_base, 0, 0
    uint4 tris[2];     // per slot: its leaf's triangles as bits of the node's triangle mask (0: inner or empty)
};
static_assert(sizeof(WideNode) == 240, "wide node is fifteen 16-byte words");

// The collapse of a binary tree (pbg_wide.cu); false when the tree does not
// fit the wide format.
bool collapse_wide(const std::vector<BvhNode>& bin, int32_t unculled, int64_t ntri, int absorb, float c_tri,
                   std::vector<WideNode>* out, std::vector<int32_t>* src);
constexpr int kWideWidth = 8;         // children per node
constexpr int kWideMaxLeaf = 7;       // triangles per leaf child
constexpr int kWideMaxOffset = 31;    // a leaf's first triangle within its node's 32
constexpr int kWideAbsorb = 4;        // subtrees of at most this many triangles may become one leaf
constexpr float kWideTriCost = 0.3f;  // a triangle test against a wide node visit

#ifdef __CUDACC__
constexpr int kWideThreads = 128;
constexpr int kWideMinBlocks = 7;  // CTAs per SM: 7 measured best of 5, 6, 7, 8
constexpr int kWideStack = 64;

// A group's entry distance kept in the upper 16 bits of a stack word,
// rounded toward -infinity (a popped group is skipped only when it lies
// beyond the hit found).
__device__ __forceinline__ uint32_t dist_bits_down(float t) {
    uint32_t b = __float_as_uint(t);
    if (b & 0x80000000u) b += 0xffffu;  // negative: a larger magnitude is smaller
    return b & 0xffff0000u;
}

// COOP (walk 6): the triangle tests of a warp's lanes spread over all 32
// lanes: lane j of round r tests pending pair r * 32 + j (pairs numbered
// lane by lane) against its owner's ray, read from shared memory; hits merge
// per owner by a 64-bit atomic maximum of hit_key (nearer t, then the larger
// index: the rule of pbrt's in-order loop that the other kernels keep too).
// It pays on incoherent batches, where a lane's pending triangles range from
// 1 to 64 (path bounces: nearest hit 1.77 -> 1.65 ms); on coherent ones the
// lanes' counts are alike and the shared-memory round trip costs more
// (camera rays 3.29 -> 4.15 ms), so the autotuner picks per batch class.

struct CoopWarp {
    float4 o[32], d[32];
    const TriRec* tris[32];      // the owner's records (scene sets)
    unsigned long long key[32];  // nearest: best hit_key (0: none); any-hit: nonzero once occluded
    float ht[32], nd[32], t[32], b1[32], b2[32];
    uint32_t m1[32], m2[32], m3[32];
    int32_t base1[32], base2[32], base3[32], off[32], occluder[32];
};

// Children in visiting order: slot ^ visit_order(octant).  Nearest hits go
// front to back; any-hit rays back to front: a shadow ray's first boxes front
// to back are the surface around its origin, which it leaves, and its
// occluders lie farther on (path frame: shadow batches 0.70 -> 0.59 ms,
// camera shadows 3.89 -> 3.50 ms).
template <bool ANY>
__device__ __forceinline__ uint32_t visit_order_of(uint32_t oct) { return ANY ? oct ^ 7u : oct; }

template <bool ANY, bool STATS, bool COOP, class Src>
__global__ void __launch_bounds__(kWideThreads, kWideMinBlocks)
    wide_walk_kernel(const Src src, int* status, unsigned long long* next, unsigned long long* wcount) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    __shared__ CoopWarp coop[COOP ? kWideThreads / 32 : 1];
    int2 stack[kWideStack];  // (child base, hits | imask << 8 | distance bits)
    int sp = 0;
    typename Src::Lane L{};
    bool has = false, exhausted = false, ok = true, fin = false;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
    RayInv ri{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float nd = 0.f;
    WalkHit h{0.f, 0.f, 0.f, -1};
    uint32_t oct = 0;
    int32_t gbase = 0;          // the current group: inner children from gbase
    uint32_t ghits = 0, gimask = 0;  // hit children in visiting order, the node's inner mask
    float gtn = 0.f;            // the group's nearest entry distance
    int32_t tbase = 0;          // pending triangles of the last node: records tbase + bit
    uint32_t tmask = 0;
    int32_t tbase2 = 0;         // a second node's triangles, found while others searched
    uint32_t tmask2 = 0;
    int32_t tbase3 = 0;         // walk 6: a third (its tests are dealt over the warp)
    uint32_t tmask3 = 0;
    int32_t rcnt = 0;           // pending degenerate records [0, rcnt)
    WorkCount wc;

    auto finish = [&]() {
        src.template store<ANY>(L, h);
        if (!ok) atomicAdd(&status[kStatusOverflow], 1);
        has = false;
        fin = true;
    };

    const int64_t n = src.count();
    for (;;) {
        fin = false;
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
                    if (!src.fetch(slot, L, o, d)) {
                        h = WalkHit{0.f, 0.f, 0.f, -1};
                        ok = true;
                        finish();  // invalid: a miss, no walk
                    } else {
                        nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
                        ri = RayInv{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
                        oct = (__float_as_uint(ri.ix) >> 31) | (__float_as_uint(ri.iy) >> 31) << 1 |
                              (__float_as_uint(ri.iz) >> 31) << 2;
                        h = WalkHit{d.w, 0.f, 0.f, -1};
                        sp = 0;
                        ok = true;
                        gbase = 0;  // the root: slot 0 of a group whose only inner child is node 0
                        gimask = 1u;
                        ghits = 1u << visit_order_of<ANY>(oct);
                        gtn = -INFINITY;
                        tmask = 0;
                        tmask2 = 0;
                        tmask3 = 0;
                        rcnt = src.unculled(L);  // degenerate records first
                        has = true;
                    }
                }
            }
        }
        if (!__any_sync(full, has)) {
            if (__all_sync(full, exhausted)) break;
            continue;
        }
        // nodes until every lane holds triangles or has ended its ray
        for (;;) {
            const bool searching = has && tmask == 0 && rcnt == 0;
            if (!__any_sync(full, searching)) break;
            // walk 6: the tests are dealt over the warp, so they need not
            // wait for the last searching lane: once four lanes hold two
            // nodes' triangles the warp tests (path frame 1,319 -> 1,436
            // Mrays/s; thresholds of 2, 3, 6, 8 lanes, or 8-20 lanes holding
            // any: 1,356-1,435)
            if (COOP && __popc(__ballot_sync(full, has && tmask2 != 0)) >= 4) break;
            // a lane that holds triangles walks on for one more node's
            // triangles (two more when the warp deals its tests over its
            // lanes) while others search, so the tests below run with fuller
            // warps (walk 6 with two more: path bounces 1.66 -> 1.64 ms)
            if (!has || (COOP ? tmask3 != 0 : tmask2 != 0) || rcnt != 0) continue;
            if (ghits != 0 && gtn > h.t) ghits = 0;  // the whole group lies beyond the hit found
            if (ghits == 0) {
                bool got = false;
                while (sp > 0) {
                    --sp;
                    const int2 e = stack[sp];
                    const float te = __uint_as_float((uint32_t)e.y & 0xffff0000u);
                    if (te <= h.t) {
                        gbase = e.x;
                        ghits = (uint32_t)e.y & 0xffu;
                        gimask = ((uint32_t)e.y >> 8) & 0xffu;
                        gtn = te;
                        got = true;
                        break;
                    }
                }
                if (!got && tmask == 0) finish();  // nothing left to walk or test
                continue;
            }
            const int pos = __ffs(ghits) - 1;
            const uint32_t rest = ghits & (ghits - 1u);
            const int cslot = pos ^ (int)visit_order_of<ANY>(oct);
            const int32_t child = gbase + __popc(gimask & ((1u << cslot) - 1u));

            const float4* np = reinterpret_cast<const float4*>(src.nodes(L) + child);
            const int4 r = __ldg(reinterpret_cast<const int4*>(np + 12));
            // the near and far planes of the ray's octant, eight slots each
            const int xo = (int)(oct & 1u) * 2, yo = 4 + (int)(oct & 2u), zo = 8 + (int)(oct & 4u) / 2;
            const float4 nx0 = __ldg(np + xo), nx1 = __ldg(np + xo + 1);
            const float4 fx0 = __ldg(np + (2 - xo)), fx1 = __ldg(np + (3 - xo));
            const float4 ny0 = __ldg(np + yo), ny1 = __ldg(np + yo + 1);
            const float4 fy0 = __ldg(np + (10 - yo)), fy1 = __ldg(np + (11 - yo));
            const float4 nz0 = __ldg(np + zo), nz1 = __ldg(np + zo + 1);
            const float4 fz0 = __ldg(np + (18 - zo)), fz1 = __ldg(np + (19 - zo));
            const float nxs[8] = {nx0.x, nx0.y, nx0.z, nx0.w, nx1.x, nx1.y, nx1.z, nx1.w};
            const float fxs[8] = {fx0.x, fx0.y, fx0.z, fx0.w, fx1.x, fx1.y, fx1.z, fx1.w};
            const float nys[8] = {ny0.x, ny0.y, ny0.z, ny0.w, ny1.x, ny1.y, ny1.z, ny1.w};
            const float fys[8] = {fy0.x, fy0.y, fy0.z, fy0.w, fy1.x, fy1.y, fy1.z, fy1.w};
            const float nzs[8] = {nz0.x, nz0.y, nz0.z, nz0.w, nz1.x, nz1.y, nz1.z, nz1.w};
            const float fzs[8] = {fz0.x, fz0.y, fz0.z, fz0.w, fz1.x, fz1.y, fz1.z, fz1.w};
            const uint4 lt0 = __ldg(reinterpret_cast<const uint4*>(np + 13));
            const uint4 lt1 = __ldg(reinterpret_cast<const uint4*>(np + 14));
            const uint32_t lts[8] = {lt0.x, lt0.y, lt0.z, lt0.w, lt1.x, lt1.y, lt1.z, lt1.w};
            const uint32_t imask = (uint32_t)r.x >> 24;
            uint32_t hits = 0, tm = 0;
            float ntn = INFINITY;  // nearest entry over the hit children: a bound for the group
#pragma unroll
            for (int k = 0; k < kWideWidth; ++k) {
                const float tnx = __fmul_rn(__fsub_rn(nxs[k], ri.ox), ri.ix);
                const float tfx = __fmul_rn(__fsub_rn(fxs[k], ri.ox), ri.ix);
                const float tny = __fmul_rn(__fsub_rn(nys[k], ri.oy), ri.iy);
                const float tfy = __fmul_rn(__fsub_rn(fys[k], ri.oy), ri.iy);
                const float tnz = __fmul_rn(__fsub_rn(nzs[k], ri.oz), ri.iz);
                const float tfz = __fmul_rn(__fsub_rn(fzs[k], ri.oz), ri.iz);
                const float tn = fmax3(tnx, tny, fmaxf(tnz, o.w));
                const float tf = fmin3(tfx, tfy, fminf(tfz, h.t));
                const bool hit = tn <= fmaf(fabsf(tf), 2.f * 3.f * 0x1p-24f / (1.f - 3.f * 0x1p-24f), tf);
                if (hit) {
                    hits |= 1u << k;
                    tm |= lts[k];
                    if (!ANY) ntn = fminf(ntn, tn);
                }
            }
            if (STATS) {
                uint32_t occupied = imask;
#pragma unroll
                for (int k = 0; k < kWideWidth; ++k) occupied |= lts[k] != 0u ? 1u << k : 0u;
                wc.node += __popc(occupied);
            }
            // hit inner children in visiting order: bit (slot ^ octant)
            uint32_t ih = hits & imask;
            const uint32_t vo = visit_order_of<ANY>(oct);
            if (vo & 1u) ih = ((ih & 0x55u) << 1) | ((ih >> 1) & 0x55u);
            if (vo & 2u) ih = ((ih & 0x33u) << 2) | ((ih >> 2) & 0x33u);
            if (vo & 4u) ih = ((ih & 0x0fu) << 4) | ((ih >> 4) & 0x0fu);
            if (ih) {
                if (rest) {
                    if (sp < kWideStack) {
                        stack[sp] = make_int2(gbase, (int)(rest | gimask << 8 | dist_bits_down(gtn)));
                        ++sp;
                    } else {
                        ok = false;
                    }
                }
                gbase = r.x & 0xffffff;
                ghits = ih;
                gimask = imask;
                gtn = ANY ? -INFINITY : ntn;
            } else {
                ghits = rest;
            }
            if (tmask == 0) {
                tbase = r.y;
                tmask = tm;
            } else if (tmask2 == 0) {
                tbase2 = r.y;
                tmask2 = tm;
            } else {
                tbase3 = r.y;
                tmask3 = tm;
            }
        }
        // the triangle tests, converged
        if (COOP) {
            // degenerate records (a ray's first round only), one lane each
            if (has && rcnt != 0) {
                const bool done = test_run<ANY, STATS>(src.tris(L), 0, rcnt, o, d, nd, h, wc);
                rcnt = 0;
                if (done) {
                    tmask = tmask2 = tmask3 = 0;
                    finish();
                }
            }
            const bool mine = has && (tmask | tmask2 | tmask3) != 0;
            const int c = mine ? __popc(tmask) + __popc(tmask2) + __popc(tmask3) : 0;
            int incl = c;
#pragma unroll
            for (int sh = 1; sh < 32; sh <<= 1) {
                const int v = __shfl_up_sync(full, incl, sh);
                if (lane >= sh) incl += v;
            }
            const int total = __shfl_sync(full, incl, 31);
            if (total > 0) {
                CoopWarp& cw = coop[threadIdx.x >> 5];
                const unsigned long long own = ANY || h.prim < 0 ? 0ull : hit_key(h.t, h.prim);
                cw.off[lane] = incl - c;
                if (mine) {
                    if (STATS) wc.leaf++;
                    cw.o[lane] = o;
                    cw.d[lane] = d;
                    if (Src::kSet) cw.tris[lane] = src.tris(L);
                    cw.nd[lane] = nd;
                    cw.ht[lane] = h.t;
                    cw.m1[lane] = tmask;
                    cw.m2[lane] = tmask2;
                    cw.m3[lane] = tmask3;
                    cw.base3[lane] = tbase3;
                    cw.base1[lane] = tbase;
                    cw.base2[lane] = tbase2;
                    cw.key[lane] = own;
                }
                __syncwarp();
                for (int g0 = 0; g0 < total; g0 += 32) {
                    const int g = g0 + lane;
                    int ci = -1;
                    unsigned long long ck = 0ull;
                    float ct = 0.f, cu1 = 0.f, cu2 = 0.f;
                    if (g < total) {
                        int i = 0;  // the owner: the last lane whose first pair is <= g
#pragma unroll
                        for (int step = 16; step; step >>= 1)
                            if (cw.off[i + step] <= g) i += step;
                        const int k = g - cw.off[i];
                        const uint32_t m1 = cw.m1[i];
                        const int n1 = __popc(m1);
                        const uint32_t m2v = cw.m2[i];
                        const int n2 = __popc(m2v);
                        const int32_t rec = k < n1        ? cw.base1[i] + (int)__fns(m1, 0, k + 1)
                                            : k < n1 + n2 ? cw.base2[i] + (int)__fns(m2v, 0, k - n1 + 1)
                                                          : cw.base3[i] + (int)__fns(cw.m3[i], 0, k - n1 - n2 + 1);
                        if (!ANY || cw.key[i] == 0ull) {
                            const float4 oo = cw.o[i], dd = cw.d[i];
                            const float bound = cw.ht[i];
                            const TriRec tr = (Src::kSet ? cw.tris[i] : src.tris(L))[rec];
                            if (STATS) wc.filt++;
                            if (pbg_filter(tr, oo, dd, cw.nd[i], bound, STATS ? &wc.filt2 : nullptr)) {
                                float tt, u1, u2;
                                if (STATS) wc.exact++;
                                if (pbg_exact_rec(tr, oo, dd, bound, &tt, &u1, &u2)) {
                                    if (STATS) wc.hit++;
                                    const int32_t id = __float_as_int(tr.c.w);
                                    if (ANY) {
                                        cw.key[i] = 1ull;
                                        cw.occluder[i] = id;
                                    } else {
                                        ci = i;
                                        ck = hit_key(tt, id);
                                        ct = tt;
                                        cu1 = u1;
                                        cu2 = u2;
                                        atomicMax(&cw.key[i], ck);
                                    }
                                }
                            }
                        }
                    }
                    __syncwarp();
                    if (!ANY && ci >= 0 && cw.key[ci] == ck) {  // this round's winner for its owner
                        cw.t[ci] = ct;
                        cw.b1[ci] = cu1;
                        cw.b2[ci] = cu2;
                    }
                    __syncwarp();
                }
                if (mine) {
                    const unsigned long long kk = cw.key[lane];
                    if (ANY) {
                        if (kk != 0ull) {
                            h.prim = cw.occluder[lane];
                            finish();
                        }
                    } else if (kk != own) {
                        h.t = cw.t[lane];
                        h.prim = key_prim(kk);
                        h.b1 = cw.b1[lane];
                        h.b2 = cw.b2[lane];
                    }
                }
                __syncwarp();
            }
            tmask = 0;
            tmask2 = 0;
            tmask3 = 0;
        } else if (has && (tmask != 0 || tmask2 != 0 || rcnt != 0)) {
            if (STATS) wc.leaf++;
            bool done = false;
            if (rcnt) {
                done = test_run<ANY, STATS>(src.tris(L), 0, rcnt, o, d, nd, h, wc);
                rcnt = 0;
            }
            while (!done && tmask) {
                const int b = __ffs(tmask) - 1;
                tmask &= tmask - 1u;
                done = test_run<ANY, STATS>(src.tris(L), tbase + b, 1, o, d, nd, h, wc);
            }
            while (!done && tmask2) {
                const int b = __ffs(tmask2) - 1;
                tmask2 &= tmask2 - 1u;
                done = test_run<ANY, STATS>(src.tris(L), tbase2 + b, 1, o, d, nd, h, wc);
            }
            tmask = 0;
            tmask2 = 0;
            if (done) finish();
        }
        if (Src::kSet) {  // completion stamps: one atomic per scene per warp
            const int sc = fin ? src.scene(L) : -1;
            const unsigned m = __match_any_sync(full, sc);
            if (fin && lane == __ffs(m) - 1) src.stamp(sc);
        }
    }
    if (STATS) wc.flush(wcount);
}


// One scene's batch: the ray-bvh walks 5 and 6.
struct SceneRays {
    static constexpr bool kSet = false;
    struct Lane {
        int64_t ray;
    };
    const WideNode* wn;
    const TriRec* wt;
    int32_t unc;
    const float4* ro;
    const float4* rd;
    const uint8_t* valid;
    const int32_t* perm;
    int64_t n;
    int32_t* prim;
    float* t;
    float* b1;
    float* b2;
    uint8_t* occ;

    __device__ __forceinline__ int64_t count() const { return n; }
    __device__ __forceinline__ bool fetch(int64_t slot, Lane& L, float4& o, float4& d) const {
        L.ray = perm ? (int64_t)perm[slot] : slot;
        if (valid != nullptr && valid[L.ray] == 0) return false;
        o = ro[L.ray];
        d = rd[L.ray];
        return true;
    }
    __device__ __forceinline__ const WideNode* nodes(const Lane&) const { return wn; }
    __device__ __forceinline__ const TriRec* tris(const Lane&) const { return wt; }
    __device__ __forceinline__ int32_t unculled(const Lane&) const { return unc; }
    template <bool ANY>
    __device__ __forceinline__ void store(const Lane& L, const WalkHit& h) const {
        if (ANY) {
            occ[L.ray] = h.prim >= 0 ? 1 : 0;
            if (prim) prim[L.ray] = h.prim;
        } else {
            const bool hit = h.prim >= 0;
            prim[L.ray] = h.prim;
            t[L.ray] = hit ? h.t : 0.f;
            b1[L.ray] = hit ? h.b1 : 0.f;
            b2[L.ray] = hit ? h.b2 : 0.f;
        }
    }
    __device__ __forceinline__ int scene(const Lane&) const { return 0; }
    __device__ __forceinline__ void stamp(int) const {}
};
#endif  // __CUDACC__

}  // namespace pbg
