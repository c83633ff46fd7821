// pbg_bvh.cu -- Accelerator "ray-bvh": rays against a SAH BVH over triangles.
//
// Replaces the fork's co-traversal kernels (bin/cl/intersection6DB_BVH.cl,
// intersection6DB_BVH2.cl, intersectionP6DB_BVH.cl: one thread per top-level
// BVH node walking the ray quadtree and the BVH subtree with a global-memory
// stack, accelerators/rayBVH.cpp:615-1323).  Here one thread owns one ray and
// walks the whole tree with a private stack, nearest child first.  Rays run
// in the caller's order (camera and shadow batches from the breadth-first
// renderer are already coherent) or, when the scene asks for it, in the
// 6-D Morton order of the per-batch ray hierarchy (pbg_rayorder.cu), which
// regroups incoherent bounce rays so the 32 rays of a warp walk nearly the
// same nodes.  Triangle records sit in leaf order, so a leaf is one
// contiguous run of 48-byte records; degenerate triangles sit in front of
// them and every ray tests them (no box bounds where pbrt's test accepts
// them).
//
// Box test: slab form with t = (bound - o) / d and the far distance widened
// by 1 + 2*gamma(3), which is conservative for the (already padded) box.
#include "pbg_internal.h"
#include "pbg_count.cuh"
#include "pbg_learn.h"
#include "pbg_tma.cuh"

namespace pbg {

constexpr int kBvhThreads = 128;
constexpr int kStackDepth = 64;

struct RayInv {
    float ox, oy, oz, ix, iy, iz;
};

__device__ __forceinline__ float safe_inv(float d) {
    float r = 1.f / d;
    return isfinite(r) ? r : copysignf(1e30f, d);
}

__device__ __forceinline__ bool slab(const RayInv& r, float lx, float hx, float ly, float hy,
                                     float lz, float hz, float tmin, float tmax, float* tnear) {
    float tx0 = (lx - r.ox) * r.ix, tx1 = (hx - r.ox) * r.ix;
    float ty0 = (ly - r.oy) * r.iy, ty1 = (hy - r.oy) * r.iy;
    float tz0 = (lz - r.oz) * r.iz, tz1 = (hz - r.oz) * r.iz;
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    *tnear = tn;
    // tf + |tf| * 2*gamma(3): each t carries at most two roundings
    return tn <= fmaf(fabsf(tf), 2.f * 3.f * 0x1p-24f / (1.f - 3.f * 0x1p-24f), tf);
}

// Tests records [start, start + cnt); returns true when an any-hit query is done.
template <bool ANY, bool STATS>
__device__ __forceinline__ bool test_run(const TriRec* __restrict__ tris, int32_t start, int32_t cnt,
                                         float4 o, float4 d, float nd, float& best_t, int32_t& best,
                                         float& bb1, float& bb2, WorkCount& wc) {
    for (int32_t k = 0; k < cnt; ++k) {
        const TriRec tr = tris[start + k];
        if (STATS) wc.filt++;
        if (!pbg_filter(tr, o, d, nd, best_t)) continue;
        float tt, u1, u2;
        if (STATS) wc.exact++;
        if (!pbg_exact_rec(tr, o, d, best_t, &tt, &u1, &u2)) continue;
        if (STATS) wc.hit++;
        const int32_t id = __float_as_int(tr.c.w);
        if (ANY) {
            best = id;
            return true;
        }
        if (tt < best_t || id > best) {
            best_t = tt;
            best = id;
            bb1 = u1;
            bb2 = u2;
        }
    }
    return false;
}

// ORDERED: pred[ray] names the cluster (a child reference cref[2k], with its
// leaf count cref[2k+1]) the learned model expects the first hit in; the
// walk visits that subtree first, then the whole tree from the root with the
// cluster skipped -- every node and leaf is still visited under the same
// t_max rule, so the result is the plain walk's.
template <bool ANY, bool STATS, bool ORDERED>
__global__ void __launch_bounds__(kBvhThreads)
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
    const float nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    const RayInv ri{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    float best_t = d.w, bb1 = 0.f, bb2 = 0.f;
    int32_t best = -1;
    bool done = unculled > 0 &&
                test_run<ANY, STATS>(tris, 0, unculled, o, d, nd, best_t, best, bb1, bb2, wc);

    int32_t stack[kStackDepth];
    float stack_t[kStackDepth];
    int sp = 0;
    int32_t node = 0;
    bool overflow = false;
    int32_t skip = INT32_MIN;  // the predicted cluster, once walked
    if (ORDERED && !done) {
        const int c = pred[ray];
        const int32_t ref = cref[2 * c], cnt = cref[2 * c + 1];
        skip = ref;
        if (ref == INT32_MIN) {
            // an unused cluster slot: plain walk
        } else if (ref < 0) {
            if (STATS) wc.leaf++;
            done = test_run<ANY, STATS>(tris, ~ref, cnt, o, d, nd, best_t, best, bb1, bb2, wc);
        } else {
            stack[sp] = 0;  // resume at the root afterwards
            stack_t[sp] = -INFINITY;
            ++sp;
            node = ref;
        }
    }
    while (!done) {
        const BvhNode nd_ = nodes[node];
        if (STATS) wc.node += 2;
        float tn0, tn1;
        bool h0 = slab(ri, nd_.n0.x, nd_.n0.y, nd_.n0.z, nd_.n0.w, nd_.n2.x, nd_.n2.y, o.w, best_t,
                       &tn0);
        bool h1 = slab(ri, nd_.n1.x, nd_.n1.y, nd_.n1.z, nd_.n1.w, nd_.n2.z, nd_.n2.w, o.w, best_t,
                       &tn1);
        const int32_t c0 = nd_.n3.x, c1 = nd_.n3.y;
        if (ORDERED) {  // the predicted cluster has been walked already
            h0 = h0 && c0 != skip;
            h1 = h1 && c1 != skip;
        }
        // Leaf children are tested at once, nearer one first.
        const bool swap = h0 && h1 && tn1 < tn0;
        for (int q = 0; q < 2 && !done; ++q) {
            const int side = swap ? 1 - q : q;
            const bool h = side == 0 ? h0 : h1;
            const int32_t c = side == 0 ? c0 : c1;
            if (!h || c >= 0) continue;
            if (STATS) wc.leaf++;
            done = test_run<ANY, STATS>(tris, ~c, side == 0 ? nd_.n3.z : nd_.n3.w, o, d, nd, best_t,
                                        best, bb1, bb2, wc);
        }
        if (done) break;
        h0 = h0 && c0 >= 0;
        h1 = h1 && c1 >= 0;
        if (h0 && h1) {
            const bool first0 = tn0 <= tn1;
            if (sp < kStackDepth) {
                stack[sp] = first0 ? c1 : c0;
                stack_t[sp] = first0 ? tn1 : tn0;
                ++sp;
            } else {
                overflow = true;
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
            if (stack_t[sp] <= best_t) {
                node = stack[sp];
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    if (overflow) atomicAdd(&status[kStatusOverflow], 1);
    if (STATS) wc.flush(wcount);
    if (ANY) {
        occ[ray] = best >= 0 ? 1 : 0;
        return;
    }
    prim_out[ray] = best;
    t_out[ray] = best >= 0 ? best_t : 0.f;
    b1_out[ray] = best >= 0 ? bb1 : 0.f;
    b2_out[ray] = best >= 0 ? bb2 : 0.f;
}

int ray_order(pbg_scene* s, const float4* o, const float4* d, int64_t n, const int32_t** perm,
              cudaStream_t st);

template <bool ANY>
static int bvh_launch(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid,
                      int64_t n, int32_t* prim, float* t, float* b1, float* b2, uint8_t* occ,
                      cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    const int32_t* perm = nullptr;
    if (s->params.ray_sort > 0) {
        int rc = ray_order(s, o, d, n, &perm, st);
        if (rc) return rc;
    }
    const uint16_t* pred = nullptr;
    const int32_t* cref = nullptr;
    int rc = learn_predict(s, o, d, n, &pred, &cref, st);
    if (rc) return rc;
    const unsigned grid = (unsigned)((n + kBvhThreads - 1) / kBvhThreads);
    const BvhNode* nodes = (const BvhNode*)s->bvh.ptr;
    const TriRec* tris = (const TriRec*)s->tris.ptr;
    int* status = (int*)s->err.ptr;
    unsigned long long* wc = (unsigned long long*)s->workc.ptr;
    prof_begin(s, st);
    if (pred) {
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
    // first-hit records for the learned ordering
    if (!ANY && s->learn && s->learn->enabled) return learn_collect(s, o, d, prim, n, st);
    return PBG_OK;
}

int bvh_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    return bvh_launch<false>(s, o, d, valid, n, prim, t, b1, b2, nullptr, st);
}

int bvh_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                 uint8_t* occ, cudaStream_t st) {
    return bvh_launch<true>(s, o, d, valid, n, nullptr, nullptr, nullptr, nullptr, occ, st);
}

}  // namespace pbg
