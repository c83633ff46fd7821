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
// (pbg_rayorder.cu).  With the learned ordering on (pbg_learn.cu) each ray
// first walks the cluster its model predicts.
#include "pbg_internal.h"
#include "pbg_learn.h"
#include "pbg_tma.cuh"
#include "pbg_walk.cuh"

namespace pbg {

constexpr int kBvhThreads = 128;

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
    WalkHit h{d.w, 0.f, 0.f, -1};
    int32_t fref = INT32_MIN, fcnt = 0;
    if (ORDERED) {
        const int c = pred[ray];
        fref = cref[2 * c];
        fcnt = cref[2 * c + 1];
    }
    const bool ok = bvh_walk<ANY, STATS, ORDERED>(nodes, tris, unculled, o, d, fref, fcnt, h, wc);
    if (!ok) atomicAdd(&status[kStatusOverflow], 1);
    if (STATS) wc.flush(wcount);
    if (ANY) {
        occ[ray] = h.prim >= 0 ? 1 : 0;
        return;
    }
    prim_out[ray] = h.prim;
    t_out[ray] = h.prim >= 0 ? h.t : 0.f;
    b1_out[ray] = h.prim >= 0 ? h.b1 : 0.f;
    b2_out[ray] = h.prim >= 0 ? h.b2 : 0.f;
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
