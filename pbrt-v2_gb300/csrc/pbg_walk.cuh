// pbg_walk.cuh -- one ray's walk through a two-wide BVH (shared by the
// ray-bvh kernels and the batched many-scene pipeline).
//
// Private stack, nearest child first, leaf children tested as soon as their
// box is hit.  Box test: slab form with t = (bound - o) / d and the far
// distance widened by 1 + 2*gamma(3), conservative for the (already padded)
// boxes.  Degenerate triangles sit in front of the leaf records and are
// tested by every ray.
#pragma once
#include "pbg_count.cuh"
#include "pbg_exact.cuh"
#include "pbg_internal.h"

namespace pbg {

#ifdef __CUDACC__

constexpr int kStackDepth = 64;

struct RayInv {
    float ox, oy, oz, ix, iy, iz;
};

__device__ __forceinline__ float safe_inv(float d) {
    float r = 1.f / d;
    return isfinite(r) ? r : copysignf(1e30f, d);
}

// Three-input max / min (one instruction on sm_100 and later); NaN inputs
// are ignored as by fmaxf / fminf.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ bool slab(const RayInv& r, float lx, float hx, float ly, float hy,
                                     float lz, float hz, float tmin, float tmax, float* tnear) {
    float tx0 = (lx - r.ox) * r.ix, tx1 = (hx - r.ox) * r.ix;
    float ty0 = (ly - r.oy) * r.iy, ty1 = (hy - r.oy) * r.iy;
    float tz0 = (lz - r.oz) * r.iz, tz1 = (hz - r.oz) * r.iz;
    float tn = fmax3(fminf(tx0, tx1), fminf(ty0, ty1), fmaxf(fminf(tz0, tz1), tmin));
    float tf = fmin3(fmaxf(tx0, tx1), fmaxf(ty0, ty1), fminf(fmaxf(tz0, tz1), tmax));
    *tnear = tn;
    // tf + |tf| * 2*gamma(3): each t carries at most two roundings
    return tn <= fmaf(fabsf(tf), 2.f * 3.f * 0x1p-24f / (1.f - 3.f * 0x1p-24f), tf);
}

// The walk's stack.  PACK: one 8-byte entry (one local load per pop) when
// the scene allows it: a child reference, with a leaf's record start (below
// 2^24) and triangle count (below 128) packed into one negative word, and
// the entry distance.  Otherwise reference, count and distance in three
// arrays.
template <bool PACK>
struct WalkStack;

template <>
struct WalkStack<true> {
    int2 e[kStackDepth];
    __device__ __forceinline__ void put(int i, int32_t ref, int32_t cnt, float t) {
        const int32_t v = ref >= 0 ? ref : (int32_t)(0x80000000u | ((uint32_t)cnt << 24) | (uint32_t)(~ref));
        e[i] = make_int2(v, __float_as_int(t));
    }
    // entry i: its distance, and (reference, count) when it is taken
    __device__ __forceinline__ float get(int i, int32_t* ref, int32_t* cnt) const {
        const int2 v = e[i];
        if (v.x >= 0) {
            *ref = v.x;
            *cnt = 0;
        } else {
            *ref = ~(int32_t)((uint32_t)v.x & 0xffffffu);
            *cnt = (int32_t)(((uint32_t)v.x >> 24) & 0x7fu);
        }
        return __int_as_float(v.y);
    }
};

template <>
struct WalkStack<false> {
    int32_t r[kStackDepth], c[kStackDepth];
    float tt[kStackDepth];
    __device__ __forceinline__ void put(int i, int32_t ref, int32_t cnt, float t) {
        r[i] = ref;
        c[i] = cnt;
        tt[i] = t;
    }
    __device__ __forceinline__ float get(int i, int32_t* ref, int32_t* cnt) const {
        *ref = r[i];
        *cnt = c[i];
        return tt[i];
    }
};

struct WalkHit {
    float t, b1, b2;
    int32_t prim;
};

// Tests records [start, start + cnt); returns true when an any-hit query is done.
template <bool ANY, bool STATS>
__device__ __forceinline__ bool test_run(const TriRec* __restrict__ tris, int32_t start, int32_t cnt,
                                         float4 o, float4 d, float nd, WalkHit& h, WorkCount& wc) {
    for (int32_t k = 0; k < cnt; ++k) {
        const TriRec tr = tris[start + k];
        if (STATS) wc.filt++;
        if (!pbg_filter(tr, o, d, nd, h.t, STATS ? &wc.filt2 : nullptr)) continue;
        float tt, u1, u2;
        if (STATS) wc.exact++;
        if (!pbg_exact_rec(tr, o, d, h.t, &tt, &u1, &u2)) continue;
        if (STATS) wc.hit++;
        const int32_t id = __float_as_int(tr.c.w);
        if (ANY) {
            h.prim = id;
            return true;
        }
        if (tt < h.t || id > h.prim) {
            h.t = tt;
            h.prim = id;
            h.b1 = u1;
            h.b2 = u2;
        }
    }
    return false;
}

// The walk.  h.t starts at the ray's maxt and h.prim at -1.  ORDERED: the
// child reference `first_ref` (a cluster the learned model picked, with leaf
// count first_cnt) is walked first and skipped later; INT32_MIN = none.
// Returns false if the private stack overflowed (the result may then miss
// hits; the caller raises the overflow status).
template <bool ANY, bool STATS, bool ORDERED>
__device__ __forceinline__ bool bvh_walk(const BvhNode* __restrict__ nodes, const TriRec* __restrict__ tris,
                                         int32_t unculled, float4 o, float4 d, int32_t first_ref,
                                         int32_t first_cnt, WalkHit& h, WorkCount& wc) {
    const float nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    const RayInv ri{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    bool done = unculled > 0 && test_run<ANY, STATS>(tris, 0, unculled, o, d, nd, h, wc);
    int2 stack[kStackDepth];  // (inner node, entry distance bits): one 8-byte entry
    int sp = 0;
    int32_t node = 0;
    bool ok = true;
    const int32_t skip = ORDERED ? first_ref : INT32_MIN;
    if (ORDERED && !done && first_ref != INT32_MIN) {
        if (first_ref < 0) {
            if (STATS) wc.leaf++;
            done = test_run<ANY, STATS>(tris, ~first_ref, first_cnt, o, d, nd, h, wc);
        } else {
            stack[sp] = make_int2(0, __float_as_int(-INFINITY));  // resume at the root afterwards
            ++sp;
            node = first_ref;
        }
    }
    while (!done) {
        const BvhNode nd_ = nodes[node];
        if (STATS) wc.node += 2;
        float tn0, tn1;
        bool h0 = slab(ri, nd_.n0.x, nd_.n0.y, nd_.n0.z, nd_.n0.w, nd_.n2.x, nd_.n2.y, o.w, h.t, &tn0);
        bool h1 = slab(ri, nd_.n1.x, nd_.n1.y, nd_.n1.z, nd_.n1.w, nd_.n2.z, nd_.n2.w, o.w, h.t, &tn1);
        const int32_t c0 = nd_.n3.x, c1 = nd_.n3.y;
        if (ORDERED) {  // the predicted cluster has been walked already
            h0 = h0 && c0 != skip;
            h1 = h1 && c1 != skip;
        }
        // Leaf children are tested at once, nearer one first.
        const bool swap = h0 && h1 && tn1 < tn0;
        for (int q = 0; q < 2 && !done; ++q) {
            const int side = swap ? 1 - q : q;
            const bool hh = side == 0 ? h0 : h1;
            const int32_t c = side == 0 ? c0 : c1;
            if (!hh || c >= 0) continue;
            if (STATS) wc.leaf++;
            done = test_run<ANY, STATS>(tris, ~c, side == 0 ? nd_.n3.z : nd_.n3.w, o, d, nd, h, wc);
        }
        if (done) break;
        h0 = h0 && c0 >= 0;
        h1 = h1 && c1 >= 0;
        if (h0 && h1) {
            const bool first0 = tn0 <= tn1;
            if (sp < kStackDepth) {
                stack[sp] = make_int2(first0 ? c1 : c0, __float_as_int(first0 ? tn1 : tn0));
                ++sp;
            } else {
                ok = false;
            }
            node = first0 ? c0 : c1;
            continue;
        }
        if (h0 || h1) {
            node = h0 ? c0 : c1;
            continue;
        }
        bool found = false;
        while (sp > 0) {
            --sp;
            const int2 e = stack[sp];
            if (__int_as_float(e.y) <= h.t) {
                node = e.x;
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    return ok;
}

#endif  // __CUDACC__

}  // namespace pbg
