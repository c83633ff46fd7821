// pbg_wide.cu -- ray-bvh walks 5 and 6: the binary SAH tree collapsed into
// an eight-wide tree, walked by persistent warps (walk 6: with the warp's
// triangle tests spread over all its lanes).
//
// The reference walks its two-wide GPU BVH (bvh.cpp:154-206 lays it out,
// rayBVH.cpp:615-1323 walks it).  Walking one node per step, the two-wide
// walk of incoherent bounce rays waits on a dependent node load at every
// step and spends much of its issue on per-visit control (votes, stack
// traffic, child ordering).  Eight children per node make the path from the
// root about a third as long (68 -> 21 node visits per ray on the
// 1,024,000-triangle path scene, every box the ray meets), and the eight box
// tests of one node are independent work for the scheduler.  The collapse is
// the SAH-optimal one (the dynamic programme of Ylitie, Karras and Laine,
// "Efficient incoherent ray traversal on GPUs through compressed wide BVHs",
// HPG 2017); the child boxes stay in 32-bit floats.
//
// Exactness.  The collapse keeps the binary tree's padded child boxes as
// they are and only drops inner levels, so every triangle still sits inside
// the boxes above it.  The slab test is the two-wide walk's, plane for plane
// (t = (plane - o) * inv, far distance widened by 1 + 2 gamma(3)); the near
// plane of each axis is picked by the sign of inv instead of a min/max of
// the two planes' distances, which is the same value (the rounded
// subtraction and product are monotone, and lo <= hi).  The leaf tests are
// the same exact tests, so every walk returns the same prim, t, b1, b2 or
// occlusion bit for bit.
//
// Built lazily on the first walk-5/6 batch of a scene: on the device from a
// device-built tree (pbg_wide_build.cu), else on the host (collapse_wide).
// Layout (240 bytes per
// node: per axis the eight low planes, then the eight high planes; the
// references; the slots' triangle masks):
//   * inner children of a node are contiguous from child_base, in slot
//     order; a child's index is child_base + popc(imask below its slot);
//   * the triangles of a node's leaf children are contiguous from tri_base
//     (a second copy of the records in this order, after the degenerate
//     records that every ray tests); a slot's 32-bit mask marks its leaf's
//     triangles (zero for an inner or empty slot);
//   * children sit in slots by the direction octant that meets them first
//     (a greedy assignment of child centroids to the eight octant
//     directions), so visiting slots in the order slot ^ octant walks the
//     children roughly front to back without sorting distances (any-hit
//     rays take slot ^ octant ^ 7: back to front).
// A lane reads only the near and far planes its octant needs, by address.
// Traversal state per lane: the current node group (child base, the hit
// inner children in visiting order, the group's nearest entry distance), the
// pending triangle mask of the last node, and a private stack of groups.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "pbg_wide.cuh"

namespace pbg {


namespace {


struct Item {
    int32_t ref, cnt;  // binary child reference (>= 0 inner, else ~start) and leaf count
    int32_t inner;     // an absorbed subtree's binary node (else -1)
    float lo[3], hi[3];
};

float area(const Item& it) {
    const float dx = it.hi[0] - it.lo[0], dy = it.hi[1] - it.lo[1], dz = it.hi[2] - it.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// Record range [first, first + count) of each binary node's subtree (the
// builder's leaf order keeps a subtree's records contiguous).
struct Span {
    int32_t first, count;
};

bool subtree_spans(const std::vector<BvhNode>& bin, std::vector<Span>* out) {
    out->assign(bin.size(), Span{INT32_MAX, 0});
    // children have larger indices than their parent in both builders
    for (size_t i = bin.size(); i-- > 0;) {
        const BvhNode& b = bin[i];
        const int32_t ref[2] = {b.n3.x, b.n3.y}, cnt[2] = {b.n3.z, b.n3.w};
        Span sp{INT32_MAX, 0};
        for (int c = 0; c < 2; ++c) {
            Span cs{INT32_MAX, 0};
            if (ref[c] >= 0) {
                if ((size_t)ref[c] <= i || (size_t)ref[c] >= bin.size()) return false;
                cs = (*out)[(size_t)ref[c]];
            } else if (cnt[c] > 0) {
                cs = Span{~ref[c], cnt[c]};
            }
            if (cs.count == 0) continue;
            if (sp.count > 0 && cs.first != sp.first + sp.count && sp.first != cs.first + cs.count) return false;
            sp.first = std::min(sp.first, cs.first);
            sp.count += cs.count;
        }
        (*out)[i] = sp;
    }
    return true;
}

// Child c of binary node n as an item (cnt 0 and ref < 0: an empty slot).
Item child_item(const BvhNode& b, int c) {
    Item it;
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

bool empty_item(const Item& it) { return it.ref < 0 && it.cnt == 0; }

// The SAH-optimal collapse (the dynamic programme of the compressed wide BVH
// paper, with its node and triangle costs as parameters): cost[n][j] is the
// least expected cost of binary node n's subtree when it may take j slots of
// its wide parent -- as one wide node (a visit, then its children in eight
// slots), as one leaf of all its triangles (at most `absorb`), or dissolved
// into its two children's items with k and j - k slots.
struct Plan {
    float c_node, c_tri;
    int absorb;
    std::vector<float> cost;    // [n * 9 + j], j = 1..8
    std::vector<int8_t> how;    // -1 wide node, -2 one leaf, -3 as with j - 1 slots, k >= 0: child 0 takes k
    std::vector<int8_t> split;  // [n]: child 0's slots when n is a wide node
};

// item costs in 0..8 slots (0: only an empty slot fits in none)
void item_costs(const Plan& P, const Item& it, float* c) {
    if (empty_item(it)) {
        for (int k = 0; k <= kWideWidth; ++k) c[k] = 0.f;
        return;
    }
    c[0] = INFINITY;
    const float leaf = it.ref < 0 ? P.c_tri * (float)it.cnt * area(it) : 0.f;
    for (int k = 1; k <= kWideWidth; ++k) c[k] = it.ref < 0 ? leaf : P.cost[(size_t)it.ref * 9 + (size_t)k];
}

// least cost of two children in j slots (child 0 takes *k_out of them)
float best_split(const float* ca, const float* cb, int j, int* k_out) {
    float best = INFINITY;
    int bk = -1;
    for (int k = 0; k <= j; ++k) {
        const float c = ca[k] + cb[j - k];
        if (c < best) {
            best = c;
            bk = k;
        }
    }
    *k_out = bk;
    return best;
}

void plan_collapse(const std::vector<BvhNode>& bin, const std::vector<Span>& span, Plan* P) {
    const size_t nn = bin.size();
    P->cost.assign(nn * 9, INFINITY);
    P->how.assign(nn * 9, -1);
    P->split.assign(nn, 4);
    for (size_t i = nn; i-- > 0;) {  // children after parents: bottom up
        const Item a = child_item(bin[i], 0), b = child_item(bin[i], 1);
        Item u = empty_item(a) ? b : a;
        if (!empty_item(a) && !empty_item(b))
            for (int ax = 0; ax < 3; ++ax) {
                u.lo[ax] = std::min(a.lo[ax], b.lo[ax]);
                u.hi[ax] = std::max(a.hi[ax], b.hi[ax]);
            }
        const float ar = empty_item(a) && empty_item(b) ? 0.f : area(u);
        float ca[kWideWidth + 1], cb[kWideWidth + 1];
        item_costs(*P, a, ca);
        item_costs(*P, b, cb);
        int k8 = 0;
        const float as_node = P->c_node * ar + best_split(ca, cb, kWideWidth, &k8);
        P->split[i] = (int8_t)k8;
        const float as_leaf = span[i].count <= P->absorb ? P->c_tri * (float)span[i].count * ar : INFINITY;
        float* c = &P->cost[i * 9];
        int8_t* h = &P->how[i * 9];
        int k1 = 0;
        const float s1 = best_split(ca, cb, 1, &k1);
        c[1] = as_node;
        h[1] = -1;
        if (as_leaf < c[1]) {
            c[1] = as_leaf;
            h[1] = -2;
        }
        if (s1 < c[1]) {
            c[1] = s1;
            h[1] = (int8_t)k1;
        }
        for (int j = 2; j <= kWideWidth; ++j) {
            int kj = 0;
            const float sj = best_split(ca, cb, j, &kj);
            if (sj < c[j - 1]) {
                c[j] = sj;
                h[j] = (int8_t)kj;
            } else {
                c[j] = c[j - 1];
                h[j] = -3;
            }
        }
    }
}

// The items of `it` in at most j slots, as the plan decided.
void emit(const std::vector<BvhNode>& bin, const std::vector<Span>& span, const Plan& P, const Item& it, int j,
          std::vector<Item>* out) {
    if (empty_item(it) || j < 1) return;
    if (it.ref < 0) {
        out->push_back(it);
        return;
    }
    const size_t n = (size_t)it.ref;
    int h = P.how[n * 9 + (size_t)j];
    while (h == -3) h = P.how[n * 9 + (size_t)(--j)];
    if (h == -1) {
        out->push_back(it);
    } else if (h == -2) {
        Item leaf = it;
        leaf.ref = ~span[n].first;
        leaf.cnt = span[n].count;
        leaf.inner = it.ref;
        out->push_back(leaf);
    } else {
        emit(bin, span, P, child_item(bin[n], 0), h, out);
        emit(bin, span, P, child_item(bin[n], 1), j - h, out);
    }
}

// A wide node's items for binary node n.
void node_items(const std::vector<BvhNode>& bin, const std::vector<Span>& span, const Plan& P, int32_t n,
                std::vector<Item>* out) {
    const int k = P.split[(size_t)n];
    emit(bin, span, P, child_item(bin[(size_t)n], 0), k, out);
    emit(bin, span, P, child_item(bin[(size_t)n], 1), kWideWidth - k, out);
}

// Slots by octant: the child that a ray of octant s meets first goes to
// slot s (greedy on dot(centroid - node centroid, octant direction)).
void assign_slots(const std::vector<Item>& items, int slot_of[kWideWidth]) {
    const int k = (int)items.size();
    float cmin[3], cmax[3];
    for (int a = 0; a < 3; ++a) {
        cmin[a] = INFINITY;
        cmax[a] = -INFINITY;
        for (const Item& it : items) {
            cmin[a] = std::min(cmin[a], it.lo[a]);
            cmax[a] = std::max(cmax[a], it.hi[a]);
        }
    }
    float rel[kWideWidth][3];
    for (int i = 0; i < k; ++i)
        for (int a = 0; a < 3; ++a)
            rel[i][a] = 0.5f * (items[(size_t)i].lo[a] + items[(size_t)i].hi[a]) - 0.5f * (cmin[a] + cmax[a]);
    float cost[kWideWidth * kWideWidth];  // [child * 8 + slot]
    for (int i = 0; i < kWideWidth; ++i)
        for (int sl = 0; sl < kWideWidth; ++sl) {
            float c = INFINITY;
            if (i < k) {
                c = 0.f;
                for (int a = 0; a < 3; ++a) c += (sl >> a & 1) ? -rel[i][a] : rel[i][a];
            }
            cost[i * kWideWidth + sl] = c;
        }
    // greedy: the cheapest (child, slot) pair left, ties to the first in
    // child-major order
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

}  // namespace

// The collapse: wide nodes breadth first (root 0) and, per record position
// of the wide copy, the position of that record in the binary tree's order.
// False when the tree does not fit the format (a leaf of more than 7
// triangles, a node's leaf triangles beyond offset 31, 2^24 nodes or more):
// the scene then keeps the two-wide walks.
bool collapse_wide(const std::vector<BvhNode>& bin, int32_t unculled, int64_t ntri, int absorb, float c_tri,
                   std::vector<WideNode>* out, std::vector<int32_t>* src) {
    out->clear();
    src->clear();
    if (bin.empty()) return false;
    std::vector<Span> span;
    if (!subtree_spans(bin, &span)) return false;
    Plan plan;
    plan.c_node = 1.f;
    plan.c_tri = c_tri;
    plan.absorb = std::min(absorb, kWideMaxLeaf);
    plan_collapse(bin, span, &plan);
    src->reserve((size_t)ntri);
    for (int32_t i = 0; i < unculled; ++i) src->push_back(i);
    struct Pending {
        int32_t wide, bin;
    };
    std::vector<Pending> queue{{0, 0}};
    out->resize(1);
    std::vector<Item> items;
    for (size_t head = 0; head < queue.size(); ++head) {
        const Pending pd = queue[head];
        items.clear();
        node_items(bin, span, plan, pd.bin, &items);
        if ((int)items.size() > kWideWidth) return false;
        // a node's leaf triangles fit the 32-bit triangle mask: the largest
        // absorbed subtrees go back to being inner children until they do
        int32_t leaf_tris = 0;
        for (const Item& it : items) leaf_tris += it.ref < 0 ? it.cnt : 0;
        while (leaf_tris > 32) {
            int big = -1;
            for (int i = 0; i < (int)items.size(); ++i)
                if (items[(size_t)i].inner >= 0 && (big < 0 || items[(size_t)i].cnt > items[(size_t)big].cnt)) big = i;
            if (big < 0) return false;
            leaf_tris -= items[(size_t)big].cnt;
            items[(size_t)big].ref = items[(size_t)big].inner;
            items[(size_t)big].cnt = 0;
            items[(size_t)big].inner = -1;
        }
        int slot_of[kWideWidth];
        assign_slots(items, slot_of);
        int item_at[kWideWidth];
        for (int s = 0; s < kWideWidth; ++s) item_at[s] = -1;
        for (int i = 0; i < (int)items.size(); ++i) item_at[slot_of[i]] = i;

        WideNode wn;
        memset(&wn, 0, sizeof(wn));  // an empty slot: a zero box, neither leaf nor inner child
        float* pl = reinterpret_cast<float*>(wn.plane);
        uint32_t tmask[kWideWidth];
        uint32_t imask = 0;
        const int32_t child_base = (int32_t)out->size();
        const int32_t tri_base = (int32_t)src->size();
        int32_t n_inner = 0;
        for (int s = 0; s < kWideWidth; ++s) {
            tmask[s] = 0;
            const int i = item_at[s];
            if (i < 0) continue;
            const Item& it = items[(size_t)i];
            for (int a = 0; a < 3; ++a) {
                pl[a * 16 + s] = it.lo[a];
                pl[a * 16 + 8 + s] = it.hi[a];
            }
            if (it.ref >= 0) {
                imask |= 1u << s;
                queue.push_back({child_base + n_inner, it.ref});
                ++n_inner;
            } else {
                const int32_t off = (int32_t)src->size() - tri_base;
                if (it.cnt > kWideMaxLeaf || off > kWideMaxOffset || off + it.cnt > 32) return false;
                tmask[s] = (uint32_t)(((1ull << it.cnt) - 1ull) << off);
                for (int32_t r = 0; r < it.cnt; ++r) src->push_back(~it.ref + r);
            }
        }
        out->resize(out->size() + (size_t)n_inner);
        if (out->size() >= (size_t)1 << 24) return false;  // child_base shares its word with imask
        wn.refs.x = (int32_t)((uint32_t)child_base | imask << 24);
        wn.refs.y = tri_base;
        wn.tris[0] = make_uint4(tmask[0], tmask[1], tmask[2], tmask[3]);
        wn.tris[1] = make_uint4(tmask[4], tmask[5], tmask[6], tmask[7]);
        (*out)[(size_t)pd.wide] = wn;
    }
    return (int64_t)src->size() == ntri;
}

__global__ void gather_records_kernel(const TriRec* __restrict__ in, const int32_t* __restrict__ src, int64_t n,
                                      TriRec* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[src[i]];
}

int ensure_wide(pbg_scene* s, bool* available, cudaStream_t st) {
    *available = false;
    if (s->wide_state < 0) return PBG_OK;
    if (s->wide_state > 0) {
        *available = true;
        return PBG_OK;
    }
    s->wide_state = -1;
    if (s->bvh_nodes <= 0) return PBG_OK;
    const auto t0 = std::chrono::steady_clock::now();
    int rc;
    DeviceBuffer dsrc;
    int64_t nwide = 0;
    cudaError_t e = cudaSuccess;
    if (!s->bvh_levels.empty()) {  // a tree built on the device: collapsed there
        bool fits = false;
        if ((rc = collapse_wide_device(s, &fits, dsrc, &nwide, st))) {
            release(dsrc);
            return rc;
        }
        if (!fits) {
            release(dsrc);
            return PBG_OK;
        }
    } else {  // a tree built on the host: collapsed there
        std::vector<WideNode> wn;
        std::vector<int32_t> src;
        if (!collapse_wide(s->host_nodes, s->unculled, s->ntri, kWideAbsorb, kWideTriCost, &wn, &src)) return PBG_OK;
        nwide = (int64_t)wn.size();
        if ((rc = ensure(s->wide, wn.size() * sizeof(WideNode))) ||
            (rc = ensure(dsrc, (size_t)std::max<int64_t>(s->ntri, 1) * sizeof(int32_t))))
            return rc;
        e = cudaMemcpy(s->wide.ptr, wn.data(), wn.size() * sizeof(WideNode), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && s->ntri > 0)
            e = cudaMemcpy(dsrc.ptr, src.data(), src.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && (rc = ensure(s->tris_wide, (size_t)std::max<int64_t>(s->ntri, 1) * sizeof(TriRec)))) {
        release(dsrc);
        return rc;
    }
    if (e == cudaSuccess && s->ntri > 0) {
        gather_records_kernel<<<(unsigned)((s->ntri + 255) / 256), 256, 0, st>>>(
            (const TriRec*)s->tris.ptr, (const int32_t*)dsrc.ptr, s->ntri, (TriRec*)s->tris_wide.ptr);
        e = cudaGetLastError();
        s->counters.kernel_launches += 1;
    }
    // later batches may run on other streams: the tree is complete before any of them
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    release(dsrc);
    if (e != cudaSuccess) return cuda_status(e, "wide BVH build");
    s->wide_nodes = nwide;
    s->wide_state = 1;
    s->counters.wide_nodes = (uint64_t)nwide;
    s->counters.wide_build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *available = true;
    return PBG_OK;
}

template <bool ANY, bool COOP>
int wide_launch(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, const int32_t* perm,
                int64_t n, int32_t* prim, float* t, float* b1, float* b2, uint8_t* occ, cudaStream_t st) {
    Work& w = s->work;
    int rc = ensure(w.counters, 64);
    if (rc) return rc;
    unsigned long long* next = (unsigned long long*)w.counters.ptr;
    PBG_CUDA(cudaMemsetAsync(next, 0, sizeof(unsigned long long), st));
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wide_walk_kernel<ANY, false, COOP, SceneRays>, kWideThreads, 0);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    int64_t blocks = (int64_t)std::max(per_sm, 1) * sms;
    blocks = std::min<int64_t>(blocks, (n + kWideThreads - 1) / kWideThreads);
    const bool stats = s->prof.level >= 2;
    const SceneRays src{(const WideNode*)s->wide.ptr, (const TriRec*)s->tris_wide.ptr, s->unculled, o, d, valid, perm,
                        n, prim, t, b1, b2, occ};
    auto kern = stats ? wide_walk_kernel<ANY, true, COOP, SceneRays> : wide_walk_kernel<ANY, false, COOP, SceneRays>;
    kern<<<(unsigned)blocks, kWideThreads, 0, st>>>(src, (int*)s->err.ptr, next,
                                                     stats ? (unsigned long long*)s->workc.ptr : nullptr);
    return PBG_OK;
}

int wide_nearest(pbg_scene* s, bool coop, const float4* o, const float4* d, const uint8_t* valid,
                 const int32_t* perm, int64_t n, int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    return coop ? wide_launch<false, true>(s, o, d, valid, perm, n, prim, t, b1, b2, nullptr, st)
                : wide_launch<false, false>(s, o, d, valid, perm, n, prim, t, b1, b2, nullptr, st);
}

int wide_occluded(pbg_scene* s, bool coop, const float4* o, const float4* d, const uint8_t* valid,
                  const int32_t* perm, int64_t n, int32_t* occluders, uint8_t* occ, cudaStream_t st) {
    return coop ? wide_launch<true, true>(s, o, d, valid, perm, n, occluders, nullptr, nullptr, nullptr, occ, st)
                : wide_launch<true, false>(s, o, d, valid, perm, n, occluders, nullptr, nullptr, nullptr, occ, st);
}

}  // namespace pbg
