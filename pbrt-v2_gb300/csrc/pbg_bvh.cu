// pbg_bvh.cu -- Accelerator "ray-bvh": rays against a SAH BVH over triangles.
//
// Replaces the fork's co-traversal kernels (bin/cl/intersection6DB_BVH.cl,
// intersection6DB_BVH2.cl, intersectionP6DB_BVH.cl: one thread per top-level
// BVH node walking the ray quadtree and the BVH subtree with a global-memory
// stack, accelerators/rayBVH.cpp:615-1323).  Here one thread owns one ray and
// walks the whole tree with a private stack, nearest child first; the
// per-bounce ray hierarchy (pbg_rayorder.cu) orders the rays so that the 32
// rays of a warp are neighbours in origin and direction and walk nearly the
// same nodes.  Triangle records sit in leaf order, so a leaf is one
// contiguous run of 48-byte records.
//
// Box test: slab form with t = (bound - o) / d and the far distance widened
// by 1 + 2*gamma(3), which is conservative for the (already padded) box.
#include "pbg_internal.h"
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

template <bool ANY>
__global__ void __launch_bounds__(kBvhThreads)
    bvh_kernel(const BvhNode* __restrict__ nodes, const TriRec* __restrict__ tris, int32_t unculled,
               const float4* __restrict__ ro, const float4* __restrict__ rd,
               const uint8_t* __restrict__ valid, const int32_t* __restrict__ perm, int64_t n,
               int32_t* __restrict__ prim_out, float* __restrict__ t_out,
               float* __restrict__ b1_out, float* __restrict__ b2_out, uint8_t* __restrict__ occ,
               int* status) {
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
    const float4 o = ro[ray], d = rd[ray];
    const float nd = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    RayInv ri{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    float best_t = d.w, bb1 = 0.f, bb2 = 0.f;
    int32_t best = -1;

    // Degenerate triangles: no box bounds where the exact test accepts them.
    for (int32_t k = 0; k < unculled; ++k) {
        const TriRec tr = tris[k];
        if (!pbg_filter(tr, o, d, nd, best_t)) continue;
        float tt, u1, u2;
        if (!pbg_exact_rec(tr, o, d, best_t, &tt, &u1, &u2)) continue;
        const int32_t id = __float_as_int(tr.c.w);
        if (ANY) {
            best = id;
            break;
        }
        if (tt < best_t || id > best) {
            best_t = tt;
            best = id;
            bb1 = u1;
            bb2 = u2;
        }
    }
    if (ANY && best >= 0) {
        occ[ray] = 1;
        return;
    }
    int32_t stack[kStackDepth];
    float stack_t[kStackDepth];
    int sp = 0;
    int32_t node = 0;
    bool overflow = false;
    for (;;) {
        const BvhNode nd_ = nodes[node];
        float tn0, tn1;
        bool h0 = slab(ri, nd_.n0.x, nd_.n0.y, nd_.n0.z, nd_.n0.w, nd_.n2.x, nd_.n2.y, o.w, best_t,
                       &tn0);
        bool h1 = slab(ri, nd_.n1.x, nd_.n1.y, nd_.n1.z, nd_.n1.w, nd_.n2.z, nd_.n2.w, o.w, best_t,
                       &tn1);
        int32_t c0 = nd_.n3.x, c1 = nd_.n3.y;
        // Leaf children are tested at once.
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const bool h = side == 0 ? h0 : h1;
            const int32_t c = side == 0 ? c0 : c1;
            if (!h || c >= 0) continue;
            const int32_t start = ~c, cnt = side == 0 ? nd_.n3.z : nd_.n3.w;
            for (int32_t k = 0; k < cnt; ++k) {
                const TriRec tr = tris[start + k];
                if (!pbg_filter(tr, o, d, nd, best_t)) continue;
                float tt, u1, u2;
                if (!pbg_exact_rec(tr, o, d, best_t, &tt, &u1, &u2)) continue;
                const int32_t id = __float_as_int(tr.c.w);
                if (ANY) {
                    best = id;
                    break;
                }
                if (tt < best_t || id > best) {
                    best_t = tt;
                    best = id;
                    bb1 = u1;
                    bb2 = u2;
                }
            }
            if (ANY && best >= 0) break;
        }
        if (ANY && best >= 0) break;
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
        if (h0) {
            node = c0;
            continue;
        }
        if (h1) {
            node = c1;
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

int bvh_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    const int32_t* perm = nullptr;
    int rc = ray_order(s, o, d, n, &perm, st);
    if (rc) return rc;
    prof_begin(s, st);
    bvh_kernel<false><<<(unsigned)((n + kBvhThreads - 1) / kBvhThreads), kBvhThreads, 0, st>>>(
        (const BvhNode*)s->bvh.ptr, (const TriRec*)s->tris.ptr, s->unculled, o, d, valid, perm, n, prim, t, b1,
        b2, nullptr, (int*)s->err.ptr);
    prof_end(s, st, kStageTraverse, 1);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

int bvh_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                 uint8_t* occ, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    const int32_t* perm = nullptr;
    int rc = ray_order(s, o, d, n, &perm, st);
    if (rc) return rc;
    prof_begin(s, st);
    bvh_kernel<true><<<(unsigned)((n + kBvhThreads - 1) / kBvhThreads), kBvhThreads, 0, st>>>(
        (const BvhNode*)s->bvh.ptr, (const TriRec*)s->tris.ptr, s->unculled, o, d, valid, perm, n, nullptr,
        nullptr, nullptr, nullptr, occ, (int*)s->err.ptr);
    prof_end(s, st, kStageTraverse, 1);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

}  // namespace pbg
