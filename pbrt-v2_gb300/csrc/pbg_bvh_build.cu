// pbg_bvh_build.cu -- the ray-bvh tree built on the device.
//
// The reference builds pbrt's BVHAccel on the CPU for every triangle part
// (accelerators/bvh.cpp:209-283, rayBVH.cpp:204-276).  This builder makes
// the tree of bvh_build.cpp -- binned SAH over all three axes with 32 bins,
// leaves of at most max_leaf triangles, degenerate triangles in front of the
// tree, every box padded outward the same way -- with the same split
// decisions, level by level on the GPU:
//
//   prep      per triangle: degenerate or not (the host test, in double),
//             its box and centroid; degenerate triangles first in the record
//             order, the others become build items in index order; the scene
//             bounds and the largest coordinate (the global pad)
//   split     one CTA per segment of the current level: node and centroid
//             bounds (block reduction), the leaf decision, 3 x 32 bins in
//             shared memory, the SAH sweep of each axis by one thread in the
//             host builder's float order, and a stable partition of the
//             segment's items into the other buffer; leaves write their
//             triangles' record order
//   link      a scan over the level's inner segments numbers their nodes
//             (breadth first), every segment writes its box (padded) and
//             reference into its parent's slot, and inner segments emit the
//             next level's two children
//
// The host reads one count per level.  Segments whose centroids fall into
// one bin split at the middle of their current order (the host builder
// takes a median by centroid there); the tree is otherwise the host tree,
// numbered breadth first instead of depth first.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pbg_internal.h"

namespace pbg {

int scan_counts(pbg_scene* s, uint32_t* a, int64_t m, cudaStream_t st);

namespace {

constexpr int kBins = 32;
constexpr int kBT = 256;  // threads per CTA
constexpr int kDepthLimit = 48;

struct BItem {
    float lo[3], hi[3], c[3];
    int32_t idx;
};

struct BSeg {
    int32_t begin, end, node, slot, depth;
};

struct BRes {
    int32_t leaf, mid;
    float lo[3], hi[3];
};

// Floats as unsigned keys whose order is the floats' order (for atomics).
__device__ __forceinline__ uint32_t fenc(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fdec(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// triangle_degenerate of bvh_build.cpp, in the same double arithmetic.
__device__ bool degenerate(const float* v) {
    for (int k = 0; k < 9; ++k)
        if (!isfinite(v[k])) return true;
    double e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
        e1[k] = __dsub_rn((double)v[3 + k], (double)v[k]);
        e2[k] = __dsub_rn((double)v[6 + k], (double)v[k]);
    }
    const double cx = __dsub_rn(__dmul_rn(e1[1], e2[2]), __dmul_rn(e1[2], e2[1]));
    const double cy = __dsub_rn(__dmul_rn(e1[2], e2[0]), __dmul_rn(e1[0], e2[2]));
    const double cz = __dsub_rn(__dmul_rn(e1[0], e2[1]), __dmul_rn(e1[1], e2[0]));
    const double a2 = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)), __dmul_rn(cz, cz)));
    const double l1 = __dmul_rn(__dadd_rn(__dadd_rn(fabs(e1[0]), fabs(e1[1])), fabs(e1[2])),
                                __dadd_rn(__dadd_rn(fabs(e2[0]), fabs(e2[1])), fabs(e2[2])));
    return !(a2 > __dmul_rn(0x1p-16, l1));
}

// Box::area of bvh_build.cpp.
__device__ __forceinline__ float box_area(const float* lo, const float* hi) {
    const float dx = __fsub_rn(hi[0], lo[0]), dy = __fsub_rn(hi[1], lo[1]), dz = __fsub_rn(hi[2], lo[2]);
    if (!(dx >= 0.f) || !(dy >= 0.f) || !(dz >= 0.f)) return 0.f;
    return __fmul_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dx, dz)), __fmul_rn(dy, dz)));
}

__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
    int b = (int)__fmul_rn(__fsub_rn(c, lo), scale);
    return b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
}

// The SAH sweep of one axis over its bins (counts, encoded lower and upper
// bounds), in the host builder's float order: the best cost and the last bin
// of the left side, or -1.
__device__ void sah_sweep(const uint32_t* cnt, const uint32_t (*blo)[3], const uint32_t (*bhi)[3], float* best_out,
                          int* bk_out) {
    float best = INFINITY;
    int bk = -1;
    float rarea[kBins];
    int rcnt[kBins];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    int c = 0;
    for (int k = kBins - 1; k > 0; --k) {
        if (cnt[k]) {
            for (int q = 0; q < 3; ++q) {
                lo[q] = fminf(lo[q], fdec(blo[k][q]));
                hi[q] = fmaxf(hi[q], fdec(bhi[k][q]));
            }
        }
        c += (int)cnt[k];
        rarea[k] = box_area(lo, hi);
        rcnt[k] = c;
    }
    for (int q = 0; q < 3; ++q) {
        lo[q] = INFINITY;
        hi[q] = -INFINITY;
    }
    c = 0;
    for (int k = 0; k < kBins - 1; ++k) {
        if (cnt[k]) {
            for (int q = 0; q < 3; ++q) {
                lo[q] = fminf(lo[q], fdec(blo[k][q]));
                hi[q] = fmaxf(hi[q], fdec(bhi[k][q]));
            }
        }
        c += (int)cnt[k];
        if (c == 0 || rcnt[k + 1] == 0) continue;
        const float cost =
            __fadd_rn(__fmul_rn(box_area(lo, hi), (float)c), __fmul_rn(rarea[k + 1], (float)rcnt[k + 1]));
        if (cost < best) {
            best = cost;
            bk = k;
        }
    }
    *best_out = best;
    *bk_out = bk;
}

// Degenerate flags per triangle, counted per block; scene bounds.
__global__ void prep_count_kernel(const float* __restrict__ tri9, int64_t n, uint32_t* __restrict__ counts,
                                  uint32_t* __restrict__ bounds) {
    const int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x;
    bool deg = false;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (i < n) {
        const float* v = tri9 + 9 * i;
        deg = degenerate(v);
        for (int k = 0; k < 9; ++k) {
            const float x = v[k];
            if (x == x) {
                lo[k % 3] = fminf(lo[k % 3], x);
                hi[k % 3] = fmaxf(hi[k % 3], x);
            }
        }
    }
    const int c = __syncthreads_count(deg);
    if (threadIdx.x == 0) counts[blockIdx.x] = (uint32_t)c;
    for (int a = 0; a < 3; ++a) {
        for (int off = 16; off; off >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&bounds[a], fenc(lo[a]));
            atomicMax(&bounds[3 + a], fenc(hi[a]));
        }
    }
}

// Degenerate triangles to the front of the record order, the others to
// build items, both in index order; the largest item coordinate.
__global__ void prep_scatter_kernel(const float* __restrict__ tri9, int64_t n, const uint32_t* __restrict__ offs,
                                    int32_t* __restrict__ order, BItem* __restrict__ items,
                                    uint32_t* __restrict__ gmax) {
    __shared__ uint32_t wdeg[kBT / 32];
    const int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x;
    const bool valid = i < n;
    const float* v = tri9 + 9 * (valid ? i : 0);
    const bool deg = valid && degenerate(v);
    const unsigned bd = __ballot_sync(0xffffffffu, deg), bv = __ballot_sync(0xffffffffu, valid);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wdeg[warp] = __popc(bd);
    __syncthreads();
    uint32_t before = 0;  // degenerate triangles of this block before this warp
    for (int w = 0; w < warp; ++w) before += wdeg[w];
    if (!valid) return;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t deg_rank = before + __popc(bd & lt);
    const int64_t block0 = (int64_t)blockIdx.x * kBT;
    if (deg) {
        order[offs[blockIdx.x] + deg_rank] = (int32_t)i;
        return;
    }
    // non-degenerate: position = non-degenerate triangles before this one
    const int64_t nd_before = block0 - offs[blockIdx.x] + (warp * 32 - before) + __popc(bv & ~bd & lt);
    BItem it;
    float m = 0.f;
    for (int a = 0; a < 3; ++a) {
        const float x0 = v[a], x1 = v[3 + a], x2 = v[6 + a];
        it.lo[a] = fminf(fminf(x0, x1), x2);
        it.hi[a] = fmaxf(fmaxf(x0, x1), x2);
        it.c[a] = __fmul_rn(0.5f, __fadd_rn(it.lo[a], it.hi[a]));
        m = fmaxf(m, fmaxf(fabsf(it.lo[a]), fabsf(it.hi[a])));
    }
    it.idx = (int32_t)i;
    items[nd_before] = it;
    atomicMax(gmax, __float_as_uint(m));  // non-negative floats order as their bits
}

// One CTA per segment: bounds, leaf decision, binned SAH, stable partition.
__global__ void __launch_bounds__(kBT) split_kernel(const BItem* __restrict__ in, BItem* __restrict__ out,
                                                    const BSeg* __restrict__ segs, BRes* __restrict__ res,
                                                    int32_t* __restrict__ order, int32_t unculled, int max_leaf,
                                                    int* __restrict__ max_depth) {
    __shared__ float red[kBT / 32][12];
    __shared__ float nb[6], cb[6];
    __shared__ uint32_t bcnt[3][kBins], blo[3][kBins][3], bhi[3][kBins][3];
    __shared__ float acost[3];
    __shared__ int asplit[3];
    __shared__ int s_leaf, s_axis, s_split, s_median;
    __shared__ uint32_t wl[kBT / 32], wr[kBT / 32];
    __shared__ int32_t run_l, run_r;
    const BSeg sg = segs[blockIdx.x];
    const int32_t np = sg.end - sg.begin;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) atomicMax(max_depth, sg.depth);
    // node box and centroid box
    float v[12];
    for (int a = 0; a < 3; ++a) {
        v[a] = INFINITY;
        v[3 + a] = -INFINITY;
        v[6 + a] = INFINITY;
        v[9 + a] = -INFINITY;
    }
    for (int32_t i = sg.begin + threadIdx.x; i < sg.end; i += kBT) {
        const BItem it = in[i];
        for (int a = 0; a < 3; ++a) {
            v[a] = fminf(v[a], it.lo[a]);
            v[3 + a] = fmaxf(v[3 + a], it.hi[a]);
            v[6 + a] = fminf(v[6 + a], it.c[a]);
            v[9 + a] = fmaxf(v[9 + a], it.c[a]);
        }
    }
    for (int k = 0; k < 12; ++k) {
        const bool is_min = (k % 6) < 3;
        for (int off = 16; off; off >>= 1) {
            const float o = __shfl_xor_sync(0xffffffffu, v[k], off);
            v[k] = is_min ? fminf(v[k], o) : fmaxf(v[k], o);
        }
        if (lane == 0) red[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const int k = threadIdx.x;
        const bool is_min = (k % 6) < 3;
        float r = red[0][k];
        for (int w = 1; w < kBT / 32; ++w) r = is_min ? fminf(r, red[w][k]) : fmaxf(r, red[w][k]);
        if (k < 6) nb[k] = r;
        else cb[k - 6] = r;
    }
    for (int k = threadIdx.x; k < 3 * kBins; k += kBT) {
        (&bcnt[0][0])[k] = 0u;
        for (int q = 0; q < 3; ++q) {
            (&blo[0][0][0])[3 * k + q] = 0xffffffffu;  // fenc(+inf) < this: empty bins decode to NaN-free +inf below
            (&bhi[0][0][0])[3 * k + q] = 0u;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int axis = 0;
        float ext = __fsub_rn(cb[3], cb[0]);
        for (int a = 1; a < 3; ++a)
            if (__fsub_rn(cb[3 + a], cb[a]) > ext) {
                axis = a;
                ext = __fsub_rn(cb[3 + a], cb[a]);
            }
        s_axis = axis;
        s_leaf = np <= max_leaf || !(ext > 0.f) || sg.depth >= kDepthLimit;
        s_median = 0;
        s_split = -1;
    }
    __syncthreads();
    if (!s_leaf) {
        for (int32_t i = sg.begin + threadIdx.x; i < sg.end; i += kBT) {
            const BItem it = in[i];
            for (int a = 0; a < 3; ++a) {
                const float ea = __fsub_rn(cb[3 + a], cb[a]);
                if (!(ea > 0.f)) continue;
                const int b = bin_of(it.c[a], cb[a], __fdiv_rn((float)kBins, ea));
                atomicAdd(&bcnt[a][b], 1u);
                for (int q = 0; q < 3; ++q) {
                    atomicMin(&blo[a][b][q], fenc(it.lo[q]));
                    atomicMax(&bhi[a][b][q], fenc(it.hi[q]));
                }
            }
        }
        __syncthreads();
        if (threadIdx.x < 3) {  // the SAH sweep of one axis, in the host builder's order
            const int a = threadIdx.x;
            float best = INFINITY;
            int bk = -1;
            if (__fsub_rn(cb[3 + a], cb[a]) > 0.f) sah_sweep(bcnt[a], blo[a], bhi[a], &best, &bk);
            acost[a] = best;
            asplit[a] = bk;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float best = INFINITY;
            int ba = -1, bs = -1;
            for (int a = 0; a < 3; ++a)
                if (asplit[a] >= 0 && acost[a] < best) {
                    best = acost[a];
                    ba = a;
                    bs = asplit[a];
                }
            if (bs < 0) {
                s_leaf = np <= 4 * max_leaf || sg.depth >= kDepthLimit;
                s_median = !s_leaf;
            } else {
                s_axis = ba;
                s_split = bs;
            }
        }
        __syncthreads();
    }
    if (s_leaf) {
        for (int32_t i = sg.begin + threadIdx.x; i < sg.end; i += kBT) order[unculled + i] = in[i].idx;
        if (threadIdx.x == 0) {
            BRes r;
            r.leaf = 1;
            r.mid = -1;
            for (int q = 0; q < 6; ++q) (q < 3 ? r.lo[q] : r.hi[q - 3]) = nb[q];
            res[blockIdx.x] = r;
        }
        return;
    }
    int32_t nleft;
    if (s_median) {  // centroids in one bin on every axis: split the current order in the middle
        for (int32_t i = sg.begin + threadIdx.x; i < sg.end; i += kBT) out[i] = in[i];
        nleft = np / 2;
    } else {
        const int a = s_axis, bs = s_split;
        nleft = 0;
        for (int k = 0; k <= bs; ++k) nleft += (int32_t)bcnt[a][k];
        const float scale = __fdiv_rn((float)kBins, __fsub_rn(cb[3 + a], cb[a]));
        const float lo = cb[a];
        if (threadIdx.x == 0) {
            run_l = 0;
            run_r = 0;
        }
        __syncthreads();
        for (int32_t base = sg.begin; base < sg.end; base += kBT) {
            const int32_t i = base + threadIdx.x;
            const bool valid = i < sg.end;
            BItem it;
            bool left = false;
            if (valid) {
                it = in[i];
                left = bin_of(it.c[a], lo, scale) <= bs;
            }
            const unsigned bl = __ballot_sync(0xffffffffu, valid && left);
            const unsigned br = __ballot_sync(0xffffffffu, valid && !left);
            if (lane == 0) {
                wl[warp] = __popc(bl);
                wr[warp] = __popc(br);
            }
            __syncthreads();
            uint32_t pl = 0, pr = 0, tl = 0, tr = 0;
            for (int w = 0; w < kBT / 32; ++w) {
                if (w < warp) {
                    pl += wl[w];
                    pr += wr[w];
                }
                tl += wl[w];
                tr += wr[w];
            }
            const unsigned lt = (1u << lane) - 1u;
            if (valid) {
                const int32_t dst = left ? sg.begin + run_l + (int32_t)(pl + __popc(bl & lt))
                                         : sg.begin + nleft + run_r + (int32_t)(pr + __popc(br & lt));
                out[dst] = it;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                run_l += (int32_t)tl;
                run_r += (int32_t)tr;
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        BRes r;
        r.leaf = 0;
        r.mid = sg.begin + nleft;
        for (int q = 0; q < 6; ++q) (q < 3 ? r.lo[q] : r.hi[q - 3]) = nb[q];
        res[blockIdx.x] = r;
    }
}

// The deep levels (many small segments): one warp per segment, the same
// steps as split_kernel (bounds, leaf decision, bins, SAH, stable partition)
// at warp scale.  Order-independent reductions and an in-order partition
// give split_kernel's decisions and item order.
constexpr int kWarpSegs = 8;            // segments (warps) per CTA
constexpr int64_t kWarpLevelSegs = 4096;  // levels of more segments than this

__global__ void __launch_bounds__(32 * kWarpSegs)
    split_warp_kernel(const BItem* __restrict__ in, BItem* __restrict__ out, const BSeg* __restrict__ segs,
                      BRes* __restrict__ res, int32_t* __restrict__ order, int32_t unculled, int max_leaf,
                      int* __restrict__ max_depth, int64_t nseg) {
    __shared__ uint32_t bcnt[kWarpSegs][3][kBins], blo[kWarpSegs][3][kBins][3], bhi[kWarpSegs][3][kBins][3];
    __shared__ float acost[kWarpSegs][3];
    __shared__ int asplit[kWarpSegs][3];
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t sidx = (int64_t)blockIdx.x * kWarpSegs + w;
    if (sidx >= nseg) return;  // the whole warp: this kernel synchronises warps only
    const BSeg sg = segs[sidx];
    const int32_t np = sg.end - sg.begin;
    if (lane == 0) atomicMax(max_depth, sg.depth);
    float v[12];
    for (int a = 0; a < 3; ++a) {
        v[a] = INFINITY;
        v[3 + a] = -INFINITY;
        v[6 + a] = INFINITY;
        v[9 + a] = -INFINITY;
    }
    for (int32_t i = sg.begin + lane; i < sg.end; i += 32) {
        const BItem it = in[i];
        for (int a = 0; a < 3; ++a) {
            v[a] = fminf(v[a], it.lo[a]);
            v[3 + a] = fmaxf(v[3 + a], it.hi[a]);
            v[6 + a] = fminf(v[6 + a], it.c[a]);
            v[9 + a] = fmaxf(v[9 + a], it.c[a]);
        }
    }
    for (int k = 0; k < 12; ++k) {
        const bool is_min = (k % 6) < 3;
        for (int off = 16; off; off >>= 1) {
            const float o = __shfl_xor_sync(full, v[k], off);
            v[k] = is_min ? fminf(v[k], o) : fmaxf(v[k], o);
        }
    }
    const float* nb = v;      // node box: lo[3], hi[3]
    const float* cb = v + 6;  // centroid box: lo[3], hi[3]
    int axis = 0;
    float ext = __fsub_rn(cb[3], cb[0]);
    for (int a = 1; a < 3; ++a)
        if (__fsub_rn(cb[3 + a], cb[a]) > ext) {
            axis = a;
            ext = __fsub_rn(cb[3 + a], cb[a]);
        }
    bool leaf = np <= max_leaf || !(ext > 0.f) || sg.depth >= kDepthLimit;
    bool median = false;
    int split = -1;
    if (!leaf) {
        for (int k = lane; k < 3 * kBins; k += 32) {
            (&bcnt[w][0][0])[k] = 0u;
            for (int q = 0; q < 3; ++q) {
                (&blo[w][0][0][0])[3 * k + q] = 0xffffffffu;
                (&bhi[w][0][0][0])[3 * k + q] = 0u;
            }
        }
        __syncwarp();
        for (int32_t i = sg.begin + lane; i < sg.end; i += 32) {
            const BItem it = in[i];
            for (int a = 0; a < 3; ++a) {
                const float ea = __fsub_rn(cb[3 + a], cb[a]);
                if (!(ea > 0.f)) continue;
                const int b = bin_of(it.c[a], cb[a], __fdiv_rn((float)kBins, ea));
                atomicAdd(&bcnt[w][a][b], 1u);
                for (int q = 0; q < 3; ++q) {
                    atomicMin(&blo[w][a][b][q], fenc(it.lo[q]));
                    atomicMax(&bhi[w][a][b][q], fenc(it.hi[q]));
                }
            }
        }
        __syncwarp();
        if (lane < 3) {
            const int a = lane;
            float best = INFINITY;
            int bk = -1;
            if (__fsub_rn(cb[3 + a], cb[a]) > 0.f) sah_sweep(bcnt[w][a], blo[w][a], bhi[w][a], &best, &bk);
            acost[w][a] = best;
            asplit[w][a] = bk;
        }
        __syncwarp();
        float best = INFINITY;
        int ba = -1, bs = -1;
        for (int a = 0; a < 3; ++a)
            if (asplit[w][a] >= 0 && acost[w][a] < best) {
                best = acost[w][a];
                ba = a;
                bs = asplit[w][a];
            }
        if (bs < 0) {
            leaf = np <= 4 * max_leaf || sg.depth >= kDepthLimit;
            median = !leaf;
        } else {
            axis = ba;
            split = bs;
        }
    }
    if (leaf) {
        for (int32_t i = sg.begin + lane; i < sg.end; i += 32) order[unculled + i] = in[i].idx;
        if (lane == 0) {
            BRes r;
            r.leaf = 1;
            r.mid = -1;
            for (int q = 0; q < 6; ++q) (q < 3 ? r.lo[q] : r.hi[q - 3]) = nb[q];
            res[sidx] = r;
        }
        return;
    }
    int32_t nleft = 0;
    if (median) {
        for (int32_t i = sg.begin + lane; i < sg.end; i += 32) out[i] = in[i];
        nleft = np / 2;
    } else {
        for (int k = 0; k <= split; ++k) nleft += (int32_t)bcnt[w][axis][k];
        const float scale = __fdiv_rn((float)kBins, __fsub_rn(cb[3 + axis], cb[axis]));
        const float lo = cb[axis];
        int32_t run_l = 0, run_r = 0;
        const unsigned lt = (1u << lane) - 1u;
        for (int32_t base = sg.begin; base < sg.end; base += 32) {
            const int32_t i = base + lane;
            const bool valid = i < sg.end;
            BItem it;
            bool left = false;
            if (valid) {
                it = in[i];
                left = bin_of(it.c[axis], lo, scale) <= split;
            }
            const unsigned bl = __ballot_sync(full, valid && left);
            const unsigned br = __ballot_sync(full, valid && !left);
            if (valid) {
                const int32_t dst = left ? sg.begin + run_l + __popc(bl & lt)
                                         : sg.begin + nleft + run_r + __popc(br & lt);
                out[dst] = it;
            }
            run_l += __popc(bl);
            run_r += __popc(br);
        }
    }
    if (lane == 0) {
        BRes r;
        r.leaf = 0;
        r.mid = sg.begin + nleft;
        for (int q = 0; q < 6; ++q) (q < 3 ? r.lo[q] : r.hi[q - 3]) = nb[q];
        res[sidx] = r;
    }
}

// ---------------------------------------------------------------------
// The top levels (a few segments holding most of the items): several CTAs
// per segment, each over a chunk of kChunk items, with the segment's bounds
// and bins merged in global memory by atomics.  Every reduction is
// order-independent and the partition stable (each chunk's left and right
// items land after those of the chunks before it, in order), so the split
// decisions and the item order equal those of split_kernel.
constexpr int kChunk = 4096;             // items per CTA
constexpr int kBigLevelSegs = 32;        // levels of at most this many segments ...
constexpr int64_t kBigItems = 1 << 17;   // ... in scenes of at least this many items

struct SegAcc {
    uint32_t box[12];  // encoded: node lo (min), node hi (max), centroid lo (min), centroid hi (max)
    uint32_t cnt[3][kBins];
    uint32_t lo[3][kBins][3], hi[3][kBins][3];
    int32_t leaf, median, axis, split, nleft;
};

__device__ __forceinline__ bool chunk_of(const BSeg& sg, int32_t* b0, int32_t* b1) {
    *b0 = sg.begin + (int32_t)blockIdx.x * kChunk;
    *b1 = min(sg.end, *b0 + kChunk);
    return *b0 < sg.end;
}

// The leaf decision of split_kernel from the segment's centroid box.
__device__ __forceinline__ bool seg_leaf(const BSeg& sg, const float* cb, int max_leaf, int* axis) {
    int ax = 0;
    float ext = __fsub_rn(cb[3], cb[0]);
    for (int a = 1; a < 3; ++a)
        if (__fsub_rn(cb[3 + a], cb[a]) > ext) {
            ax = a;
            ext = __fsub_rn(cb[3 + a], cb[a]);
        }
    *axis = ax;
    return (sg.end - sg.begin) <= max_leaf || !(ext > 0.f) || sg.depth >= kDepthLimit;
}

__global__ void big_init_kernel(SegAcc* __restrict__ acc) {
    SegAcc& A = acc[blockIdx.x];
    for (int k = threadIdx.x; k < 12; k += blockDim.x) A.box[k] = (k % 6) < 3 ? 0xffffffffu : 0u;
    for (int k = threadIdx.x; k < 3 * kBins; k += blockDim.x) {
        (&A.cnt[0][0])[k] = 0u;
        for (int q = 0; q < 3; ++q) {
            (&A.lo[0][0][0])[3 * k + q] = 0xffffffffu;
            (&A.hi[0][0][0])[3 * k + q] = 0u;
        }
    }
}

__global__ void __launch_bounds__(kBT) big_bounds_kernel(const BItem* __restrict__ in, const BSeg* __restrict__ segs,
                                                         SegAcc* __restrict__ acc, int* __restrict__ max_depth) {
    __shared__ float red[kBT / 32][12];
    const BSeg sg = segs[blockIdx.y];
    int32_t b0, b1;
    if (!chunk_of(sg, &b0, &b1)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicMax(max_depth, sg.depth);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float v[12];
    for (int a = 0; a < 3; ++a) {
        v[a] = INFINITY;
        v[3 + a] = -INFINITY;
        v[6 + a] = INFINITY;
        v[9 + a] = -INFINITY;
    }
    for (int32_t i = b0 + threadIdx.x; i < b1; i += kBT) {
        const BItem it = in[i];
        for (int a = 0; a < 3; ++a) {
            v[a] = fminf(v[a], it.lo[a]);
            v[3 + a] = fmaxf(v[3 + a], it.hi[a]);
            v[6 + a] = fminf(v[6 + a], it.c[a]);
            v[9 + a] = fmaxf(v[9 + a], it.c[a]);
        }
    }
    for (int k = 0; k < 12; ++k) {
        const bool is_min = (k % 6) < 3;
        for (int off = 16; off; off >>= 1) {
            const float o = __shfl_xor_sync(0xffffffffu, v[k], off);
            v[k] = is_min ? fminf(v[k], o) : fmaxf(v[k], o);
        }
        if (lane == 0) red[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const int k = threadIdx.x;
        const bool is_min = (k % 6) < 3;
        float r = red[0][k];
        for (int w = 1; w < kBT / 32; ++w) r = is_min ? fminf(r, red[w][k]) : fmaxf(r, red[w][k]);
        if (is_min)
            atomicMin(&acc[blockIdx.y].box[k], fenc(r));
        else
            atomicMax(&acc[blockIdx.y].box[k], fenc(r));
    }
}

__global__ void __launch_bounds__(kBT) big_bins_kernel(const BItem* __restrict__ in, const BSeg* __restrict__ segs,
                                                       SegAcc* __restrict__ acc, int max_leaf) {
    __shared__ uint32_t bcnt[3][kBins], blo[3][kBins][3], bhi[3][kBins][3];
    const BSeg sg = segs[blockIdx.y];
    int32_t b0, b1;
    if (!chunk_of(sg, &b0, &b1)) return;
    SegAcc& A = acc[blockIdx.y];
    float cb[6];
    for (int k = 0; k < 6; ++k) cb[k] = fdec(A.box[6 + k]);
    int axis;
    if (seg_leaf(sg, cb, max_leaf, &axis)) return;  // the same for every CTA of the segment
    for (int k = threadIdx.x; k < 3 * kBins; k += kBT) {
        (&bcnt[0][0])[k] = 0u;
        for (int q = 0; q < 3; ++q) {
            (&blo[0][0][0])[3 * k + q] = 0xffffffffu;
            (&bhi[0][0][0])[3 * k + q] = 0u;
        }
    }
    __syncthreads();
    for (int32_t i = b0 + threadIdx.x; i < b1; i += kBT) {
        const BItem it = in[i];
        for (int a = 0; a < 3; ++a) {
            const float ea = __fsub_rn(cb[3 + a], cb[a]);
            if (!(ea > 0.f)) continue;
            const int b = bin_of(it.c[a], cb[a], __fdiv_rn((float)kBins, ea));
            atomicAdd(&bcnt[a][b], 1u);
            for (int q = 0; q < 3; ++q) {
                atomicMin(&blo[a][b][q], fenc(it.lo[q]));
                atomicMax(&bhi[a][b][q], fenc(it.hi[q]));
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * kBins; k += kBT) {
        const int a = k / kBins, b = k % kBins;
        if (bcnt[a][b] == 0u) continue;
        atomicAdd(&A.cnt[a][b], bcnt[a][b]);
        for (int q = 0; q < 3; ++q) {
            atomicMin(&A.lo[a][b][q], blo[a][b][q]);
            atomicMax(&A.hi[a][b][q], bhi[a][b][q]);
        }
    }
}

// One warp per segment: split_kernel's leaf decision and SAH choice from the
// merged bins; the segment's result.
__global__ void big_decide_kernel(const BSeg* __restrict__ segs, SegAcc* __restrict__ acc, BRes* __restrict__ res,
                                  int max_leaf) {
    __shared__ float acost[3];
    __shared__ int asplit[3];
    const BSeg sg = segs[blockIdx.x];
    SegAcc& A = acc[blockIdx.x];
    float nb[6], cb[6];
    for (int k = 0; k < 6; ++k) {
        nb[k] = fdec(A.box[k]);
        cb[k] = fdec(A.box[6 + k]);
    }
    int axis;
    const bool leaf0 = seg_leaf(sg, cb, max_leaf, &axis);
    if (!leaf0 && threadIdx.x < 3) {
        const int a = threadIdx.x;
        float best = INFINITY;
        int bk = -1;
        if (__fsub_rn(cb[3 + a], cb[a]) > 0.f) sah_sweep(A.cnt[a], A.lo[a], A.hi[a], &best, &bk);
        acost[a] = best;
        asplit[a] = bk;
    }
    __syncwarp();
    if (threadIdx.x != 0) return;
    const int32_t np = sg.end - sg.begin;
    int leaf = leaf0, median = 0, split = -1;
    if (!leaf) {
        float best = INFINITY;
        int ba = -1, bs = -1;
        for (int a = 0; a < 3; ++a)
            if (asplit[a] >= 0 && acost[a] < best) {
                best = acost[a];
                ba = a;
                bs = asplit[a];
            }
        if (bs < 0) {
            leaf = np <= 4 * max_leaf || sg.depth >= kDepthLimit;
            median = !leaf;
        } else {
            axis = ba;
            split = bs;
        }
    }
    int32_t nleft = 0;
    if (!leaf) {
        if (median) {
            nleft = np / 2;
        } else {
            for (int k = 0; k <= split; ++k) nleft += (int32_t)A.cnt[axis][k];
        }
    }
    A.leaf = leaf;
    A.median = median;
    A.axis = axis;
    A.split = split;
    A.nleft = nleft;
    BRes r;
    r.leaf = leaf;
    r.mid = leaf ? -1 : sg.begin + nleft;
    for (int q = 0; q < 6; ++q) (q < 3 ? r.lo[q] : r.hi[q - 3]) = nb[q];
    res[blockIdx.x] = r;
}

// Leaves write their record order, median splits copy their items; splits by
// bin count each chunk's left items.
__global__ void __launch_bounds__(kBT) big_count_kernel(const BItem* __restrict__ in, BItem* __restrict__ out,
                                                        const BSeg* __restrict__ segs, const SegAcc* __restrict__ acc,
                                                        int32_t* __restrict__ order, int32_t unculled,
                                                        uint32_t* __restrict__ lcnt, int64_t chunks) {
    const BSeg sg = segs[blockIdx.y];
    int32_t b0, b1;
    if (!chunk_of(sg, &b0, &b1)) return;
    const SegAcc& A = acc[blockIdx.y];
    if (A.leaf) {
        for (int32_t i = b0 + threadIdx.x; i < b1; i += kBT) order[unculled + i] = in[i].idx;
        return;
    }
    if (A.median) {
        for (int32_t i = b0 + threadIdx.x; i < b1; i += kBT) out[i] = in[i];
        return;
    }
    const int a = A.axis;
    const float lo = fdec(A.box[6 + a]);
    const float scale = __fdiv_rn((float)kBins, __fsub_rn(fdec(A.box[9 + a]), lo));
    uint32_t c = 0;
    for (int32_t base = b0; base < b1; base += kBT) {
        const int32_t i = base + threadIdx.x;
        const bool left = i < b1 && bin_of(in[i].c[a], lo, scale) <= A.split;
        c += (uint32_t)__syncthreads_count(left);
    }
    if (threadIdx.x == 0) lcnt[(int64_t)blockIdx.y * chunks + blockIdx.x] = c;
}

// The stable partition of split segments: each chunk's left items after the
// left items of the chunks before it, its right items likewise after nleft.
__global__ void __launch_bounds__(kBT) big_scatter_kernel(const BItem* __restrict__ in, BItem* __restrict__ out,
                                                          const BSeg* __restrict__ segs,
                                                          const SegAcc* __restrict__ acc,
                                                          const uint32_t* __restrict__ lcnt, int64_t chunks) {
    __shared__ uint32_t wl[kBT / 32], wr[kBT / 32];
    __shared__ int32_t run_l, run_r;
    const BSeg sg = segs[blockIdx.y];
    int32_t b0, b1;
    if (!chunk_of(sg, &b0, &b1)) return;
    const SegAcc& A = acc[blockIdx.y];
    if (A.leaf || A.median) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        int32_t pl = 0;
        for (unsigned k = 0; k < blockIdx.x; ++k) pl += (int32_t)lcnt[(int64_t)blockIdx.y * chunks + k];
        run_l = pl;
        run_r = (b0 - sg.begin) - pl;
    }
    __syncthreads();
    const int a = A.axis;
    const float lo = fdec(A.box[6 + a]);
    const float scale = __fdiv_rn((float)kBins, __fsub_rn(fdec(A.box[9 + a]), lo));
    const int32_t nleft = A.nleft;
    for (int32_t base = b0; base < b1; base += kBT) {
        const int32_t i = base + threadIdx.x;
        const bool valid = i < b1;
        BItem it;
        bool left = false;
        if (valid) {
            it = in[i];
            left = bin_of(it.c[a], lo, scale) <= A.split;
        }
        const unsigned bl = __ballot_sync(0xffffffffu, valid && left);
        const unsigned br = __ballot_sync(0xffffffffu, valid && !left);
        if (lane == 0) {
            wl[warp] = __popc(bl);
            wr[warp] = __popc(br);
        }
        __syncthreads();
        uint32_t pl = 0, pr = 0, tl = 0, tr = 0;
        for (int w = 0; w < kBT / 32; ++w) {
            if (w < warp) {
                pl += wl[w];
                pr += wr[w];
            }
            tl += wl[w];
            tr += wr[w];
        }
        const unsigned lt = (1u << lane) - 1u;
        if (valid) {
            const int32_t dst = left ? sg.begin + run_l + (int32_t)(pl + __popc(bl & lt))
                                     : sg.begin + nleft + run_r + (int32_t)(pr + __popc(br & lt));
            out[dst] = it;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            run_l += (int32_t)tl;
            run_r += (int32_t)tr;
        }
        __syncthreads();
    }
}

__global__ void inner_count_kernel(const BRes* __restrict__ res, int64_t nseg, uint32_t* __restrict__ counts) {
    const int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x;
    const int c = __syncthreads_count(i < nseg && !res[i].leaf);
    if (threadIdx.x == 0) counts[blockIdx.x] = (uint32_t)c;
}

// pad_of / write_child of bvh_build.cpp, one scalar store per field (the
// two children of a node are written by different threads).
__device__ void write_slot(BvhNode* nd, int slot, const float* lo_in, const float* hi_in, int32_t child,
                           int32_t count, float gpad) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        if (count == 0 && child < 0) {
            lo[a] = INFINITY;
            hi[a] = -INFINITY;
            continue;
        }
        const float mag = fmaxf(fabsf(lo_in[a]), fabsf(hi_in[a]));
        float ext = __fsub_rn(hi_in[a], lo_in[a]);
        if (!(ext >= 0.f)) ext = 0.f;
        const float p = __fadd_rn(__fmul_rn(__fadd_rn(mag, ext), 0x1p-13f), gpad);
        lo[a] = nextafterf(__fsub_rn(lo_in[a], p), -INFINITY);
        hi[a] = nextafterf(__fadd_rn(hi_in[a], p), INFINITY);
    }
    if (slot == 0) {
        nd->n0.x = lo[0]; nd->n0.y = hi[0]; nd->n0.z = lo[1]; nd->n0.w = hi[1];
        nd->n2.x = lo[2]; nd->n2.y = hi[2];
        nd->n3.x = child; nd->n3.z = count;
    } else {
        nd->n1.x = lo[0]; nd->n1.y = hi[0]; nd->n1.z = lo[1]; nd->n1.w = hi[1];
        nd->n2.z = lo[2]; nd->n2.w = hi[2];
        nd->n3.y = child; nd->n3.w = count;
    }
}

__global__ void link_kernel(const BSeg* __restrict__ segs, const BRes* __restrict__ res, int64_t nseg,
                            const uint32_t* __restrict__ offs, int32_t node_base, BvhNode* __restrict__ nodes,
                            BSeg* __restrict__ next, int32_t unculled, const uint32_t* __restrict__ gmax) {
    __shared__ uint32_t wbase[kBT / 32];
    const int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x;
    const bool valid = i < nseg;
    const bool inner = valid && !res[i].leaf;
    const unsigned b = __ballot_sync(0xffffffffu, inner);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wbase[warp] = __popc(b);
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += wbase[w];
    if (!valid) return;
    const float m = __uint_as_float(*gmax);
    const float gpad = isfinite(m) ? __fmul_rn(m, 0x1p-18f) : 0.f;
    const BSeg sg = segs[i];
    const BRes r = res[i];
    const float empty_lo[3] = {INFINITY, INFINITY, INFINITY}, empty_hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (r.leaf) {
        const int32_t start = unculled + sg.begin, cnt = sg.end - sg.begin;
        if (sg.node < 0) {  // the whole scene in one leaf
            write_slot(&nodes[0], 0, r.lo, r.hi, ~start, cnt, gpad);
            write_slot(&nodes[0], 1, empty_lo, empty_hi, -1, 0, gpad);
        } else {
            write_slot(&nodes[sg.node], sg.slot, r.lo, r.hi, ~start, cnt, gpad);
        }
        return;
    }
    const uint32_t rank = offs[blockIdx.x] + before + __popc(b & ((1u << lane) - 1u));
    const int32_t self = node_base + (int32_t)rank;
    if (sg.node >= 0) write_slot(&nodes[sg.node], sg.slot, r.lo, r.hi, self, 0, gpad);
    next[2 * rank] = BSeg{sg.begin, r.mid, self, 0, sg.depth + 1};
    next[2 * rank + 1] = BSeg{r.mid, sg.end, self, 1, sg.depth + 1};
}

__global__ void empty_root_kernel(BvhNode* nodes) {
    const float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    write_slot(&nodes[0], 0, lo, hi, -1, 0, 0.f);
    write_slot(&nodes[0], 1, lo, hi, -1, 0, 0.f);
}

}  // namespace

// Builds s->bvh from the scene's device triangles (original order, tri9)
// and writes the record order (degenerate triangles first) into order_dev
// [ntri]; fills bvh_nodes, bvh_depth, unculled, scene_lo / scene_hi.
int build_bvh_device(pbg_scene* s, const float* tri9, int64_t ntri, int max_leaf, int32_t* order_dev,
                     cudaStream_t st) {
    if (max_leaf < 1) max_leaf = 4;
    const int64_t nb = (ntri + kBT - 1) / kBT;
    DeviceBuffer counts, small, items_a, items_b, segs_a, segs_b, res, acc, lcnt;
    struct Guard {
        DeviceBuffer* b[9];
        ~Guard() {
            for (DeviceBuffer* x : b) release(*x);
        }
    } guard{{&counts, &small, &items_a, &items_b, &segs_a, &segs_b, &res, &acc, &lcnt}};
    const size_t ni = (size_t)std::max<int64_t>(ntri, 1);
    int rc;
    if ((rc = ensure(counts, (size_t)(std::max<int64_t>(nb, ni / kBT + 1) + 8) * 4)) || (rc = ensure(small, 64)) ||
        (rc = ensure(items_a, ni * sizeof(BItem))) || (rc = ensure(items_b, ni * sizeof(BItem))) ||
        (rc = ensure(segs_a, ni * sizeof(BSeg))) || (rc = ensure(segs_b, ni * sizeof(BSeg))) ||
        (rc = ensure(res, ni * sizeof(BRes))) || (rc = ensure(s->bvh, ni * sizeof(BvhNode))))
        return rc;
    uint32_t* sm = (uint32_t*)small.ptr;  // [0..5] scene bounds, [6] gmax, [7] max depth
    std::vector<uint32_t> init = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u};
    PBG_CUDA(cudaMemcpyAsync(sm, init.data(), init.size() * 4, cudaMemcpyHostToDevice, st));
    int32_t ndeg = 0;
    if (ntri > 0) {
        uint32_t* cnt = (uint32_t*)counts.ptr;
        prep_count_kernel<<<(unsigned)nb, kBT, 0, st>>>(tri9, ntri, cnt, sm);
        PBG_CUDA(cudaGetLastError());
        uint32_t last = 0, off = 0;
        PBG_CUDA(cudaMemcpyAsync(&last, cnt + nb - 1, 4, cudaMemcpyDeviceToHost, st));
        if ((rc = scan_counts(s, cnt, nb, st))) return rc;
        PBG_CUDA(cudaMemcpyAsync(&off, cnt + nb - 1, 4, cudaMemcpyDeviceToHost, st));
        prep_scatter_kernel<<<(unsigned)nb, kBT, 0, st>>>(tri9, ntri, cnt, order_dev, (BItem*)items_a.ptr, sm + 6);
        PBG_CUDA(cudaGetLastError());
        PBG_CUDA(cudaStreamSynchronize(st));
        ndeg = (int32_t)(off + last);
        s->counters.kernel_launches += 2;
    }
    const int64_t nitems = ntri - ndeg;
    BvhNode* nodes = (BvhNode*)s->bvh.ptr;
    int32_t node_base = 0;
    s->bvh_levels.clear();
    if (nitems == 0) {
        empty_root_kernel<<<1, 1, 0, st>>>(nodes);
        PBG_CUDA(cudaGetLastError());
        node_base = 1;
    } else {
        BSeg root{0, (int32_t)nitems, -1, 0, 0};
        PBG_CUDA(cudaMemcpyAsync(segs_a.ptr, &root, sizeof(root), cudaMemcpyHostToDevice, st));
        BItem* in = (BItem*)items_a.ptr;
        BItem* out = (BItem*)items_b.ptr;
        BSeg* cur = (BSeg*)segs_a.ptr;
        BSeg* nxt = (BSeg*)segs_b.ptr;
        int64_t nseg = 1;
        while (nseg > 0) {
            if (nseg <= kBigLevelSegs && nitems >= kBigItems) {  // the top levels: several CTAs per segment
                const int64_t chunks = (nitems + kChunk - 1) / kChunk;
                if ((rc = ensure(acc, (size_t)nseg * sizeof(SegAcc))) ||
                    (rc = ensure(lcnt, (size_t)(nseg * chunks) * sizeof(uint32_t))))
                    return rc;
                SegAcc* A = (SegAcc*)acc.ptr;
                const dim3 g((unsigned)chunks, (unsigned)nseg);
                big_init_kernel<<<(unsigned)nseg, kBT, 0, st>>>(A);
                big_bounds_kernel<<<g, kBT, 0, st>>>(in, cur, A, (int*)(sm + 7));
                big_bins_kernel<<<g, kBT, 0, st>>>(in, cur, A, max_leaf);
                big_decide_kernel<<<(unsigned)nseg, 32, 0, st>>>(cur, A, (BRes*)res.ptr, max_leaf);
                big_count_kernel<<<g, kBT, 0, st>>>(in, out, cur, A, order_dev, ndeg, (uint32_t*)lcnt.ptr, chunks);
                big_scatter_kernel<<<g, kBT, 0, st>>>(in, out, cur, A, (const uint32_t*)lcnt.ptr, chunks);
                s->counters.kernel_launches += 5;
            } else if (nseg > kWarpLevelSegs) {  // the deep levels: a warp per segment
                split_warp_kernel<<<(unsigned)((nseg + kWarpSegs - 1) / kWarpSegs), 32 * kWarpSegs, 0, st>>>(
                    in, out, cur, (BRes*)res.ptr, order_dev, ndeg, max_leaf, (int*)(sm + 7), nseg);
            } else {
                split_kernel<<<(unsigned)nseg, kBT, 0, st>>>(in, out, cur, (BRes*)res.ptr, order_dev, ndeg,
                                                            max_leaf, (int*)(sm + 7));
            }
            PBG_CUDA(cudaGetLastError());
            const int64_t lb = (nseg + kBT - 1) / kBT;
            uint32_t* cnt = (uint32_t*)counts.ptr;
            inner_count_kernel<<<(unsigned)lb, kBT, 0, st>>>((const BRes*)res.ptr, nseg, cnt);
            PBG_CUDA(cudaGetLastError());
            uint32_t last = 0, off = 0;
            PBG_CUDA(cudaMemcpyAsync(&last, cnt + lb - 1, 4, cudaMemcpyDeviceToHost, st));
            if ((rc = scan_counts(s, cnt, lb, st))) return rc;
            PBG_CUDA(cudaMemcpyAsync(&off, cnt + lb - 1, 4, cudaMemcpyDeviceToHost, st));
            link_kernel<<<(unsigned)lb, kBT, 0, st>>>(cur, (const BRes*)res.ptr, nseg, cnt, node_base, nodes, nxt,
                                                      ndeg, sm + 6);
            PBG_CUDA(cudaGetLastError());
            PBG_CUDA(cudaStreamSynchronize(st));
            s->counters.kernel_launches += 3;
            const int64_t inner = (int64_t)off + last;
            if (inner > 0) {
                s->bvh_levels.push_back(node_base);
                s->bvh_levels.push_back((int32_t)inner);
            }
            node_base += (int32_t)inner;
            if (node_base == 0) node_base = 1;  // the root was a leaf
            nseg = 2 * inner;
            std::swap(in, out);
            std::swap(cur, nxt);
        }
    }
    uint32_t h[8];
    PBG_CUDA(cudaMemcpyAsync(h, sm, sizeof(h), cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    auto dec = [](uint32_t u) {
        const uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
        float f;
        memcpy(&f, &b, 4);
        return f;
    };
    for (int a = 0; a < 3; ++a) {
        s->scene_lo[a] = ntri > 0 ? dec(h[a]) : 0.f;
        s->scene_hi[a] = ntri > 0 ? dec(h[3 + a]) : 0.f;
    }
    if (s->bvh_levels.empty()) s->bvh_levels = {0, 1};  // one root node: a leaf, or no triangles
    s->bvh_nodes = node_base;
    s->bvh_depth = (int)h[7];
    s->unculled = ndeg;
    s->counters.bvh_nodes = (uint64_t)node_base;
    return PBG_OK;
}

}  // namespace pbg
