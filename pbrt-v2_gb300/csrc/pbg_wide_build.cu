// pbg_wide_build.cu -- the eight-wide tree collapsed on the device from a
// device-built two-wide tree (the same collapse as collapse_wide in
// pbg_wide.cu, decision for decision: the same float operations, rounded the
// same way, so both give the same nodes).
//
//   plan   bottom up, one launch per level of the two-wide tree (the device
//          builder numbers it breadth first and records its levels): per
//          node its subtree's record span and the SAH costs of the collapse
//          -- as one wide node, as one leaf, or dissolved into its children's
//          items -- in 1..8 slots of its parent
//   emit   top down, one launch per level of the wide tree: per wide node its
//          items as the plan decided (at most eight), slots by the octant
//          that meets each child first, counts of inner children and leaf
//          triangles
//   write  after a scan of both counts: the node, the next level's list of
//          (wide node, two-wide node) pairs, and per record position of the
//          wide copy the record's position in the two-wide order
// The host reads two totals per wide level.  Every write index is checked
// against its buffer; a tree that does not fit the wide format (or a check
// that fails) sets a flag and the scene keeps the two-wide walks.
#include <algorithm>
#include <vector>

#include "pbg_wide.cuh"

namespace pbg {

int scan_counts(pbg_scene* s, uint32_t* a, int64_t m, cudaStream_t st);

namespace {

constexpr int kWT = 128;
constexpr int kEmitStack = 24;
constexpr float kNodeCost = 1.f;

struct DItem {
    int32_t ref, cnt, inner;  // two-wide reference (>= 0 inner, else ~start), leaf count, absorbed node
    float lo[3], hi[3];
};

__device__ __forceinline__ bool d_empty(const DItem& it) { return it.ref < 0 && it.cnt == 0; }

// (hi - lo) products in the host collapse's order: dx*dy + dy*dz, then + dz*dx
__device__ __forceinline__ float d_area(const DItem& it) {
    const float dx = __fsub_rn(it.hi[0], it.lo[0]), dy = __fsub_rn(it.hi[1], it.lo[1]);
    const float dz = __fsub_rn(it.hi[2], it.lo[2]);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
}

__device__ __forceinline__ DItem d_child(const BvhNode& b, int c) {
    DItem it;
    it.ref = c == 0 ? b.n3.x : b.n3.y;
    it.cnt = it.ref >= 0 ? 0 : (c == 0 ? b.n3.z : b.n3.w);
    it.inner = -1;
    const float4 box = c == 0 ? b.n0 : b.n1;
    it.lo[0] = box.x;
    it.hi[0] = box.y;
    it.lo[1] = box.z;
    it.hi[1] = box.w;
    it.lo[2] = c == 0 ? b.n2.x : b.n2.z;
    it.hi[2] = c == 0 ? b.n2.y : b.n2.w;
    return it;
}

__device__ __forceinline__ void d_item_costs(const DItem& it, const float* __restrict__ cost, float c_tri,
                                             float* c) {
    if (d_empty(it)) {
#pragma unroll
        for (int k = 0; k <= kWideWidth; ++k) c[k] = 0.f;
        return;
    }
    c[0] = INFINITY;
    const float leaf = it.ref < 0 ? __fmul_rn(__fmul_rn(c_tri, (float)it.cnt), d_area(it)) : 0.f;
#pragma unroll
    for (int k = 1; k <= kWideWidth; ++k) c[k] = it.ref < 0 ? leaf : cost[(int64_t)it.ref * 9 + k];
}

__device__ __forceinline__ float d_best_split(const float* ca, const float* cb, int j, int* k_out) {
    float best = INFINITY;
    int bk = -1;
    for (int k = 0; k <= j; ++k) {
        const float c = __fadd_rn(ca[k], cb[j - k]);
        if (c < best) {
            best = c;
            bk = k;
        }
    }
    *k_out = bk;
    return best;
}

// The plan for the nodes [first, first + count) of one level.
__global__ void wide_plan_kernel(const BvhNode* __restrict__ bin, int32_t nnodes, int32_t first, int32_t count,
                                 float* cost, int8_t* how, int8_t* split, int32_t* sfirst, int32_t* scount,
                                 float c_tri, int absorb, int* fail) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int32_t n = first + (int32_t)i;
    const BvhNode b = bin[n];
    const DItem a = d_child(b, 0), c = d_child(b, 1);
    // the subtree's record span (children: larger numbers, already planned)
    int32_t f = INT32_MAX, k = 0;
    bool ok = true;
    for (int ch = 0; ch < 2; ++ch) {
        const DItem& it = ch == 0 ? a : c;
        int32_t cf = INT32_MAX, ck = 0;
        if (it.ref >= 0) {
            if (it.ref <= n || it.ref >= nnodes) {
                ok = false;
                continue;
            }
            cf = sfirst[it.ref];
            ck = scount[it.ref];
        } else if (it.cnt > 0) {
            cf = ~it.ref;
            ck = it.cnt;
        }
        if (ck == 0) continue;
        if (k > 0 && cf != f + k && f != cf + ck) ok = false;
        f = min(f, cf);
        k += ck;
    }
    if (!ok) {
        atomicExch(fail, 1);
        return;
    }
    sfirst[n] = f;
    scount[n] = k;
    DItem u = d_empty(a) ? c : a;
    if (!d_empty(a) && !d_empty(c))
        for (int ax = 0; ax < 3; ++ax) {
            u.lo[ax] = c.lo[ax] < a.lo[ax] ? c.lo[ax] : a.lo[ax];
            u.hi[ax] = a.hi[ax] < c.hi[ax] ? c.hi[ax] : a.hi[ax];
        }
    const float ar = d_empty(a) && d_empty(c) ? 0.f : d_area(u);
    float ca[kWideWidth + 1], cb[kWideWidth + 1];
    d_item_costs(a, cost, c_tri, ca);
    d_item_costs(c, cost, c_tri, cb);
    int k8 = 0;
    const float as_node = __fadd_rn(__fmul_rn(kNodeCost, ar), d_best_split(ca, cb, kWideWidth, &k8));
    split[n] = (int8_t)k8;
    const float as_leaf = k <= absorb ? __fmul_rn(__fmul_rn(c_tri, (float)k), ar) : INFINITY;
    float* cn = cost + (int64_t)n * 9;
    int8_t* hn = how + (int64_t)n * 9;
    cn[0] = INFINITY;
    hn[0] = -1;
    int k1 = 0;
    const float s1 = d_best_split(ca, cb, 1, &k1);
    float c1 = as_node;
    int8_t h1 = -1;
    if (as_leaf < c1) {
        c1 = as_leaf;
        h1 = -2;
    }
    if (s1 < c1) {
        c1 = s1;
        h1 = (int8_t)k1;
    }
    cn[1] = c1;
    hn[1] = h1;
    float prev = c1;
    for (int j = 2; j <= kWideWidth; ++j) {
        int kj = 0;
        const float sj = d_best_split(ca, cb, j, &kj);
        if (sj < prev) {
            cn[j] = sj;
            hn[j] = (int8_t)kj;
            prev = sj;
        } else {
            cn[j] = prev;
            hn[j] = -3;
        }
    }
}

// Slots by octant (the host collapse's greedy assignment, same float order).
__device__ void d_assign_slots(const DItem* items, int k, int* slot_of) {
    float cmin[3], cmax[3];
    for (int a = 0; a < 3; ++a) {
        cmin[a] = INFINITY;
        cmax[a] = -INFINITY;
        for (int i = 0; i < k; ++i) {
            cmin[a] = items[i].lo[a] < cmin[a] ? items[i].lo[a] : cmin[a];
            cmax[a] = cmax[a] < items[i].hi[a] ? items[i].hi[a] : cmax[a];
        }
    }
    float rel[kWideWidth][3];
    for (int i = 0; i < k; ++i)
        for (int a = 0; a < 3; ++a)
            rel[i][a] = __fsub_rn(__fmul_rn(0.5f, __fadd_rn(items[i].lo[a], items[i].hi[a])),
                                  __fmul_rn(0.5f, __fadd_rn(cmin[a], cmax[a])));
    float cost[kWideWidth * kWideWidth];
    for (int i = 0; i < kWideWidth; ++i)
        for (int sl = 0; sl < kWideWidth; ++sl) {
            float c = INFINITY;
            if (i < k) {
                c = 0.f;
                for (int a = 0; a < 3; ++a) c = __fadd_rn(c, (sl >> a & 1) ? -rel[i][a] : rel[i][a]);
            }
            cost[i * kWideWidth + sl] = c;
        }
    for (int i = 0; i < kWideWidth; ++i) slot_of[i] = -1;
    for (int round = 0; round < k; ++round) {
        int best = 0;
        float bv = cost[0];
        for (int t = 1; t < kWideWidth * kWideWidth; ++t) {
            const bool lt = cost[t] < bv;
            bv = lt ? cost[t] : bv;
            best = lt ? t : best;
        }
        const int i = best / kWideWidth, sl = best % kWideWidth;
        slot_of[i] = sl;
        for (int q = 0; q < kWideWidth; ++q) {
            cost[i * kWideWidth + q] = INFINITY;
            cost[q * kWideWidth + sl] = INFINITY;
        }
    }
}

// Per wide node of the level: its items in slot order (ref -1, cnt 0 for an
// empty slot), inner children and leaf triangles.
__global__ void wide_emit_kernel(const BvhNode* __restrict__ bin, const int2* __restrict__ list, int32_t m,
                                 const int8_t* __restrict__ how, const int8_t* __restrict__ split,
                                 const int32_t* __restrict__ sfirst, const int32_t* __restrict__ scount,
                                 DItem* scratch, uint32_t* n_inner, uint32_t* n_tris, int* fail) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t n = list[i].y;
    DItem items[kWideWidth];
    int ni = 0;
    struct Pend {
        DItem it;
        int j;
    };
    Pend stack[kEmitStack];
    int sp = 0;
    bool ok = true;
    const BvhNode b = bin[n];
    const int k0 = split[n];
    stack[sp++] = Pend{d_child(b, 1), kWideWidth - k0};
    stack[sp++] = Pend{d_child(b, 0), k0};
    while (sp > 0 && ok) {
        const Pend p = stack[--sp];
        int j = p.j;
        if (d_empty(p.it) || j < 1) continue;
        if (p.it.ref < 0) {
            if (ni >= kWideWidth) ok = false;
            else items[ni++] = p.it;
            continue;
        }
        const int32_t c = p.it.ref;
        int h = how[(int64_t)c * 9 + j];
        while (h == -3 && j > 1) h = how[(int64_t)c * 9 + (--j)];
        if (h == -1 || h == -2) {
            if (ni >= kWideWidth) {
                ok = false;
                continue;
            }
            DItem it = p.it;
            if (h == -2) {  // the subtree as one leaf
                it.ref = ~sfirst[c];
                it.cnt = scount[c];
                it.inner = c;
            }
            items[ni++] = it;
        } else if (h >= 0 && sp + 2 <= kEmitStack) {
            const BvhNode cb = bin[c];
            stack[sp++] = Pend{d_child(cb, 1), j - h};
            stack[sp++] = Pend{d_child(cb, 0), h};
        } else {
            ok = false;
        }
    }
    // the node's leaf triangles fit the 32-bit mask: the largest absorbed
    // subtrees go back to being inner children until they do
    int32_t leaf_tris = 0;
    for (int q = 0; q < ni; ++q) leaf_tris += items[q].ref < 0 ? items[q].cnt : 0;
    while (ok && leaf_tris > 32) {
        int big = -1;
        for (int q = 0; q < ni; ++q)
            if (items[q].inner >= 0 && (big < 0 || items[q].cnt > items[big].cnt)) big = q;
        if (big < 0) {
            ok = false;
            break;
        }
        leaf_tris -= items[big].cnt;
        items[big].ref = items[big].inner;
        items[big].cnt = 0;
        items[big].inner = -1;
    }
    int slot_of[kWideWidth];
    if (ok) d_assign_slots(items, ni, slot_of);
    DItem* out = scratch + i * kWideWidth;
    for (int sl = 0; sl < kWideWidth; ++sl) {
        out[sl].ref = -1;
        out[sl].cnt = 0;
        out[sl].inner = -1;
    }
    uint32_t inner = 0, tris = 0;
    if (ok)
        for (int q = 0; q < ni; ++q) {
            const int sl = slot_of[q];
            if (sl < 0 || sl >= kWideWidth) {
                ok = false;
                break;
            }
            out[sl] = items[q];
            if (items[q].ref >= 0) {
                ++inner;
            } else {
                if (items[q].cnt > kWideMaxLeaf) ok = false;
                tris += (uint32_t)items[q].cnt;
            }
        }
    if (tris > 32) ok = false;
    if (!ok) {
        atomicExch(fail, 1);
        inner = tris = 0;
    }
    n_inner[i] = inner;
    n_tris[i] = tris;
}

// The level's nodes, the next level's list and the record map, after the
// exclusive scans of the counts.
__global__ void wide_write_kernel(const int2* __restrict__ list, int32_t m, const DItem* __restrict__ scratch,
                                  const uint32_t* __restrict__ inner_off, const uint32_t* __restrict__ tri_off,
                                  int32_t next_start, int32_t cursor, WideNode* wide, int32_t cap_nodes,
                                  int2* next, int32_t* src, int32_t ntri, int* fail) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t w = list[i].x;
    const int32_t child_base = next_start + (int32_t)inner_off[i];
    const int32_t tri_base = cursor + (int32_t)tri_off[i];
    const DItem* it = scratch + i * kWideWidth;
    WideNode node;
    float* pl = reinterpret_cast<float*>(node.plane);
    uint32_t masks[kWideWidth];
    uint32_t imask = 0;
    int32_t rank = 0, off = 0;
    bool ok = w >= 0 && w < cap_nodes;
    for (int sl = 0; sl < kWideWidth; ++sl) {
        masks[sl] = 0;
        const bool empty = d_empty(it[sl]);
        for (int a = 0; a < 3; ++a) {
            pl[a * 16 + sl] = empty ? 0.f : it[sl].lo[a];
            pl[a * 16 + 8 + sl] = empty ? 0.f : it[sl].hi[a];
        }
        if (empty) continue;
        if (it[sl].ref >= 0) {
            imask |= 1u << sl;
            const int32_t cw = child_base + rank;
            const int32_t at = (int32_t)inner_off[i] + rank;
            if (cw < cap_nodes && at < cap_nodes) next[at] = make_int2(cw, it[sl].ref);
            else ok = false;
            ++rank;
        } else {
            const int32_t cnt = it[sl].cnt;
            const int32_t first = ~it[sl].ref;
            if (off + cnt > 32 || tri_base + off + cnt > ntri || first < 0 || first + cnt > ntri) {
                ok = false;
                continue;
            }
            masks[sl] = (uint32_t)(((1ull << cnt) - 1ull) << off);
            for (int32_t r = 0; r < cnt; ++r) src[tri_base + off + r] = first + r;
            off += cnt;
        }
    }
    if (child_base + rank > cap_nodes || child_base >= (1 << 24)) ok = false;
    if (!ok) {
        atomicExch(fail, 1);
        return;
    }
    node.refs = make_int4((int32_t)((uint32_t)child_base | imask << 24), tri_base, 0, 0);
    node.tris[0] = make_uint4(masks[0], masks[1], masks[2], masks[3]);
    node.tris[1] = make_uint4(masks[4], masks[5], masks[6], masks[7]);
    wide[w] = node;
}

__global__ void wide_iota_kernel(int32_t* src, int32_t n) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) src[i] = i;
}

}  // namespace

int collapse_wide_device(pbg_scene* s, bool* fits, DeviceBuffer& src, int64_t* nwide, cudaStream_t st) {
    *fits = false;
    *nwide = 0;
    const int32_t nn = (int32_t)s->bvh_nodes;
    const std::vector<int32_t>& lv = s->bvh_levels;
    if (nn <= 0 || lv.size() < 2) return PBG_OK;
    const int64_t ntri = s->ntri;
    int rc;
    DeviceBuffer cost, how, split, sfirst, scount, flag, la, lb, scratch, ci, ct;
    auto done = [&](int code) {
        DeviceBuffer* all[] = {&cost, &how, &split, &sfirst, &scount, &flag, &la, &lb, &scratch, &ci, &ct};
        for (DeviceBuffer* b : all) release(*b);
        return code;
    };
    if ((rc = ensure(cost, (size_t)nn * 9 * sizeof(float))) || (rc = ensure(how, (size_t)nn * 9)) ||
        (rc = ensure(split, (size_t)nn)) || (rc = ensure(sfirst, (size_t)nn * 4)) ||
        (rc = ensure(scount, (size_t)nn * 4)) || (rc = ensure(flag, 16)) ||
        (rc = ensure(la, (size_t)nn * sizeof(int2))) || (rc = ensure(lb, (size_t)nn * sizeof(int2))) ||
        (rc = ensure(s->wide, (size_t)nn * sizeof(WideNode))) ||
        (rc = ensure(src, (size_t)std::max<int64_t>(ntri, 1) * sizeof(int32_t))))
        return done(rc);
    int* fail = (int*)flag.ptr;
    if (cudaMemsetAsync(fail, 0, 16, st) != cudaSuccess) return done(cuda_status(cudaGetLastError(), "memset"));
    const BvhNode* bin = (const BvhNode*)s->bvh.ptr;
    for (size_t l = lv.size() / 2; l-- > 0;) {  // bottom up
        const int32_t first = lv[2 * l], count = lv[2 * l + 1];
        if (count <= 0 || first < 0 || (int64_t)first + count > nn) return done(PBG_OK);
        wide_plan_kernel<<<(unsigned)((count + kWT - 1) / kWT), kWT, 0, st>>>(
            bin, nn, first, count, (float*)cost.ptr, (int8_t*)how.ptr, (int8_t*)split.ptr, (int32_t*)sfirst.ptr,
            (int32_t*)scount.ptr, kWideTriCost, kWideAbsorb, fail);
        s->counters.kernel_launches += 1;
    }
    PBG_CUDA(cudaGetLastError());
    {  // a tree the plan rejected is not walked further
        int h_fail = 0;
        PBG_CUDA(cudaMemcpyAsync(&h_fail, fail, 4, cudaMemcpyDeviceToHost, st));
        PBG_CUDA(cudaStreamSynchronize(st));
        if (h_fail) return done(PBG_OK);
    }
    if (s->unculled > 0) {
        wide_iota_kernel<<<(unsigned)((s->unculled + 255) / 256), 256, 0, st>>>((int32_t*)src.ptr, s->unculled);
        s->counters.kernel_launches += 1;
    }
    const int2 root = make_int2(0, 0);
    PBG_CUDA(cudaMemcpyAsync(la.ptr, &root, sizeof(root), cudaMemcpyHostToDevice, st));
    int2* cur = (int2*)la.ptr;
    int2* nxt = (int2*)lb.ptr;
    int64_t m = 1, next_start = 1, cursor = s->unculled;
    while (m > 0) {
        if ((rc = ensure(scratch, (size_t)m * kWideWidth * sizeof(DItem))) ||
            (rc = ensure(ci, (size_t)m * 4 + 16)) || (rc = ensure(ct, (size_t)m * 4 + 16)))
            return done(rc);
        uint32_t* c_in = (uint32_t*)ci.ptr;
        uint32_t* c_tr = (uint32_t*)ct.ptr;
        const unsigned g = (unsigned)((m + kWT - 1) / kWT);
        wide_emit_kernel<<<g, kWT, 0, st>>>(bin, cur, (int32_t)m, (const int8_t*)how.ptr, (const int8_t*)split.ptr,
                                            (const int32_t*)sfirst.ptr, (const int32_t*)scount.ptr,
                                            (DItem*)scratch.ptr, c_in, c_tr, fail);
        PBG_CUDA(cudaGetLastError());
        uint32_t last[2] = {0, 0}, off[2] = {0, 0};
        PBG_CUDA(cudaMemcpyAsync(&last[0], c_in + m - 1, 4, cudaMemcpyDeviceToHost, st));
        PBG_CUDA(cudaMemcpyAsync(&last[1], c_tr + m - 1, 4, cudaMemcpyDeviceToHost, st));
        if ((rc = scan_counts(s, c_in, m, st)) || (rc = scan_counts(s, c_tr, m, st))) return done(rc);
        PBG_CUDA(cudaMemcpyAsync(&off[0], c_in + m - 1, 4, cudaMemcpyDeviceToHost, st));
        PBG_CUDA(cudaMemcpyAsync(&off[1], c_tr + m - 1, 4, cudaMemcpyDeviceToHost, st));
        PBG_CUDA(cudaStreamSynchronize(st));
        const int64_t tot_inner = (int64_t)off[0] + last[0], tot_tris = (int64_t)off[1] + last[1];
        if (next_start + tot_inner > nn || cursor + tot_tris > ntri) return done(PBG_OK);  // cannot happen
        wide_write_kernel<<<g, kWT, 0, st>>>(cur, (int32_t)m, (const DItem*)scratch.ptr, c_in, c_tr,
                                             (int32_t)next_start, (int32_t)cursor, (WideNode*)s->wide.ptr, nn, nxt,
                                             (int32_t*)src.ptr, (int32_t)ntri, fail);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 8;
        next_start += tot_inner;
        cursor += tot_tris;
        m = tot_inner;
        std::swap(cur, nxt);
    }
    int h_fail = 0;
    PBG_CUDA(cudaMemcpyAsync(&h_fail, fail, 4, cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    if (h_fail == 0 && cursor == ntri) {
        *fits = true;
        *nwide = next_start;
    }
    return done(PBG_OK);
}

}  // namespace pbg
