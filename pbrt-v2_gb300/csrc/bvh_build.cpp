// bvh_build.cpp -- SAH BVH over the scene's triangles, built on the host when
// the scene is created, for Accelerator "ray-bvh".
//
// The reference builds pbrt's BVHAccel per triangle part on the CPU
// (accelerators/bvh.cpp:209-283 with gpu=true, flattened breadth-first by
// GPUbufferWide, bvh.cpp:154-206, into 32-byte GPUNode records,
// accelerators/bvh.h:75-79).  Here one binned-SAH tree (32 bins on each
// axis, leaves of at most 4 triangles) covers the whole scene (no
// 60k-triangle parts) and is stored as two-wide nodes that carry
// both children's boxes (BvhNode, 64 bytes), which halves the dependent node
// fetches of a traversal step.
//
// Every box is padded outward: by 2^-13 of its own magnitude and extent, and
// by 2^-18 of the scene's largest coordinate.  The exact triangle test can
// accept a ray that meets the triangle's plane slightly outside the triangle
// (its barycentric rounding); the padding keeps such triangles inside their
// boxes so that culling never removes a hit the exact test would report.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "pbg_internal.h"

namespace pbg {

namespace {

struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int a = 0; a < 3; ++a) {
            lo[a] = INFINITY;
            hi[a] = -INFINITY;
        }
    }
    void grow(const Box& b) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow(const float p[3]) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    float area() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.f) || !(dy >= 0.f) || !(dz >= 0.f)) return 0.f;
        return 2.f * (dx * dy + dx * dz + dy * dz);
    }
};

struct Item {
    Box box;
    float c[3];
    int32_t idx;
};

struct Task {
    int32_t node;  // node index to fill, or -1 for the root
    int32_t slot;  // 0/1: which child slot of `node`
    int32_t begin, end, depth;
};

constexpr int kBins = 32;

float pad_of(float lo, float hi, float global_pad) {
    float mag = std::max(std::fabs(lo), std::fabs(hi));
    float ext = hi - lo;
    if (!(ext >= 0.f)) ext = 0.f;
    return (mag + ext) * 0x1p-13f + global_pad;
}

void write_child(BvhNode& n, int slot, const Box& b, int32_t child, int32_t count,
                 float global_pad) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        if (count == 0 && child < 0) {  // empty slot: a box no ray meets
            lo[a] = INFINITY;
            hi[a] = -INFINITY;
            continue;
        }
        float p = pad_of(b.lo[a], b.hi[a], global_pad);
        lo[a] = nextafterf(b.lo[a] - p, -INFINITY);
        hi[a] = nextafterf(b.hi[a] + p, INFINITY);
    }
    if (slot == 0) {
        n.n0 = make_float4(lo[0], hi[0], lo[1], hi[1]);
        n.n2.x = lo[2];
        n.n2.y = hi[2];
        n.n3.x = child;
        n.n3.z = count;
    } else {
        n.n1 = make_float4(lo[0], hi[0], lo[1], hi[1]);
        n.n2.z = lo[2];
        n.n2.w = hi[2];
        n.n3.y = child;
        n.n3.w = count;
    }
}

}  // namespace

bool triangle_degenerate(const float* v) {
    for (int k = 0; k < 9; ++k)
        if (!std::isfinite(v[k])) return true;
    double e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
        e1[k] = (double)v[3 + k] - v[k];
        e2[k] = (double)v[6 + k] - v[k];
    }
    const double cx = e1[1] * e2[2] - e1[2] * e2[1];
    const double cy = e1[2] * e2[0] - e1[0] * e2[2];
    const double cz = e1[0] * e2[1] - e1[1] * e2[0];
    const double a2 = std::sqrt(cx * cx + cy * cy + cz * cz);
    const double l1 = (std::fabs(e1[0]) + std::fabs(e1[1]) + std::fabs(e1[2])) *
                      (std::fabs(e2[0]) + std::fabs(e2[1]) + std::fabs(e2[2]));
    return !(a2 > 0x1p-16 * l1);
}

void build_bvh(const float* tri9, int64_t ntri, int max_leaf, HostBvh* out) {
    out->nodes.clear();
    out->order.clear();
    out->max_depth = 0;
    out->unculled = 0;
    if (max_leaf < 1) max_leaf = 4;
    // Degenerate triangles first: they are tested by every ray, outside the tree.
    for (int64_t i = 0; i < ntri; ++i)
        if (triangle_degenerate(tri9 + 9 * i)) out->order.push_back((int32_t)i);
    out->unculled = (int32_t)out->order.size();
    std::vector<Item> items;
    items.reserve((size_t)(ntri - out->unculled));
    float gmax = 0.f;
    for (int64_t i = 0; i < ntri; ++i) {
        if (triangle_degenerate(tri9 + 9 * i)) continue;
        items.emplace_back();
        Item& it = items.back();
        it.box.reset();
        for (int v = 0; v < 3; ++v) it.box.grow(tri9 + 9 * i + 3 * v);
        for (int a = 0; a < 3; ++a) {
            it.c[a] = 0.5f * (it.box.lo[a] + it.box.hi[a]);
            gmax = std::max(gmax, std::max(std::fabs(it.box.lo[a]), std::fabs(it.box.hi[a])));
        }
        it.idx = (int32_t)i;
    }
    const float global_pad = std::isfinite(gmax) ? gmax * 0x1p-18f : 0.f;

    BvhNode root{};
    out->nodes.push_back(root);
    const int64_t nitems = (int64_t)items.size();
    if (nitems == 0) {
        Box e;
        e.reset();
        write_child(out->nodes[0], 0, e, -1, 0, global_pad);
        write_child(out->nodes[0], 1, e, -1, 0, global_pad);
        return;
    }
    // The root node's two slots hold the two halves of the first split (or
    // one leaf and an empty slot when everything fits one leaf).
    std::vector<Task> stack;
    stack.push_back({-1, 0, 0, (int32_t)nitems, 0});
    std::vector<int32_t>& order = out->order;
    order.reserve((size_t)ntri);

    while (!stack.empty()) {
        Task tk = stack.back();
        stack.pop_back();
        Box nb, cb;
        nb.reset();
        cb.reset();
        for (int32_t i = tk.begin; i < tk.end; ++i) {
            nb.grow(items[i].box);
            cb.grow(items[i].c);
        }
        const int32_t np = tk.end - tk.begin;
        int axis = 0;
        float ext = cb.hi[0] - cb.lo[0];
        for (int a = 1; a < 3; ++a)
            if (cb.hi[a] - cb.lo[a] > ext) {
                axis = a;
                ext = cb.hi[a] - cb.lo[a];
            }
        int32_t mid = -1;
        bool leaf = np <= max_leaf || !(ext > 0.f) || tk.depth >= 48;
        if (!leaf) {
            // binned SAH over every axis with a centroid extent; the lowest
            // cost wins
            float best = INFINITY;
            int best_axis = -1, best_split = -1;
            for (int a = 0; a < 3; ++a) {
                const float ea = cb.hi[a] - cb.lo[a];
                if (!(ea > 0.f)) continue;
                int cnt[kBins] = {0};
                Box bb[kBins];
                for (int k = 0; k < kBins; ++k) bb[k].reset();
                const float scale = kBins / ea;
                for (int32_t i = tk.begin; i < tk.end; ++i) {
                    int b = (int)((items[i].c[a] - cb.lo[a]) * scale);
                    b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                    cnt[b]++;
                    bb[b].grow(items[i].box);
                }
                float rarea[kBins];
                int rcnt[kBins];
                Box acc;
                acc.reset();
                int c = 0;
                for (int k = kBins - 1; k > 0; --k) {
                    acc.grow(bb[k]);
                    c += cnt[k];
                    rarea[k] = acc.area();
                    rcnt[k] = c;
                }
                acc.reset();
                c = 0;
                for (int k = 0; k < kBins - 1; ++k) {
                    acc.grow(bb[k]);
                    c += cnt[k];
                    if (c == 0 || rcnt[k + 1] == 0) continue;
                    const float cost = acc.area() * c + rarea[k + 1] * rcnt[k + 1];
                    if (cost < best) {
                        best = cost;
                        best_axis = a;
                        best_split = k;
                    }
                }
            }
            if (best_split < 0) {
                leaf = np <= 4 * max_leaf || tk.depth >= 48;
                if (!leaf) {  // centroids collapse into one bin: median split
                    mid = tk.begin + np / 2;
                    std::nth_element(items.begin() + tk.begin, items.begin() + mid,
                                     items.begin() + tk.end, [axis](const Item& x, const Item& y) {
                                         return x.c[axis] < y.c[axis];
                                     });
                }
            } else {
                const int a = best_axis;
                const float scale = kBins / (cb.hi[a] - cb.lo[a]);
                const float lo = cb.lo[a];
                auto it = std::partition(items.begin() + tk.begin, items.begin() + tk.end,
                                         [&](const Item& x) {
                                             int b = (int)((x.c[a] - lo) * scale);
                                             b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                                             return b <= best_split;
                                         });
                mid = (int32_t)(it - items.begin());
                if (mid == tk.begin || mid == tk.end) mid = tk.begin + np / 2;
            }
        }
        out->max_depth = std::max(out->max_depth, tk.depth);
        if (leaf) {
            const int32_t start = (int32_t)order.size();
            for (int32_t i = tk.begin; i < tk.end; ++i) order.push_back(items[i].idx);
            if (tk.node < 0) {  // whole scene in one leaf
                write_child(out->nodes[0], 0, nb, ~start, np, global_pad);
                Box e;
                e.reset();
                write_child(out->nodes[0], 1, e, -1, 0, global_pad);
            } else {
                write_child(out->nodes[tk.node], tk.slot, nb, ~start, np, global_pad);
            }
            continue;
        }
        int32_t self;
        if (tk.node < 0) {
            self = 0;
        } else {
            self = (int32_t)out->nodes.size();
            out->nodes.push_back(BvhNode{});
            write_child(out->nodes[tk.node], tk.slot, nb, self, 0, global_pad);
        }
        // Right half first so the left half is processed (and numbered) next.
        stack.push_back({self, 1, mid, tk.end, tk.depth + 1});
        stack.push_back({self, 0, tk.begin, mid, tk.depth + 1});
    }
}

}  // namespace pbg

namespace pbg {

// Triangles in clusters of kClusterTris consecutive records, built top down
// like a SAH tree whose splits may only fall on whole clusters: each part is
// sorted by centroid along each axis, and the split (an axis and a multiple
// of kClusterTris) that minimises the children's bounding-box areas weighted
// by their triangle counts is taken, until a part holds one cluster.  Every
// cluster but the last is full and compact in space (its bounding sphere
// about 0.55 of that of 32 consecutive Morton codes on the terrain scene),
// so the rayhierarchy's cluster tests cull more, and neighbouring records
// stay neighbours in space.
void cluster_triangle_order(const float* tri9, int64_t ntri, std::vector<int32_t>* order) {
    order->resize((size_t)ntri);
    if (ntri == 0) return;
    std::vector<float> c((size_t)ntri * 3);
    std::vector<Box> box((size_t)ntri);
    for (int64_t i = 0; i < ntri; ++i) {
        const float* v = tri9 + 9 * i;
        Box& b = box[(size_t)i];
        b.reset();
        for (int a = 0; a < 3; ++a) {
            float x = (v[a] + v[3 + a] + v[6 + a]) * (1.f / 3.f);
            if (!std::isfinite(x)) x = 0.f;
            c[3 * i + a] = x;
            for (int k = 0; k < 3; ++k) {
                const float w = v[3 * k + a];
                if (std::isfinite(w)) {
                    b.lo[a] = std::min(b.lo[a], w);
                    b.hi[a] = std::max(b.hi[a], w);
                }
            }
        }
    }
    std::vector<int32_t>& o = *order;
    for (int64_t i = 0; i < ntri; ++i) o[(size_t)i] = (int32_t)i;
    std::vector<int32_t> sorted[3];
    std::vector<float> right;  // suffix areas at the candidate splits
    struct Part {
        int64_t begin, end;
    };
    std::vector<Part> stack;
    stack.push_back({0, ntri});
    while (!stack.empty()) {
        const Part p = stack.back();
        stack.pop_back();
        const int64_t np = p.end - p.begin;
        if (np <= kClusterTris) continue;
        const int64_t nsplit = (np - 1) / kClusterTris;  // splits at k * kClusterTris, k = 1..nsplit
        double best = INFINITY;
        int best_axis = 0;
        int64_t best_at = kClusterTris;
        for (int a = 0; a < 3; ++a) {
            std::vector<int32_t>& srt = sorted[a];
            srt.assign(o.begin() + p.begin, o.begin() + p.end);
            std::sort(srt.begin(), srt.end(), [&](int32_t x, int32_t y) {
                const float cx = c[3 * (size_t)x + a], cy = c[3 * (size_t)y + a];
                return cx < cy || (cx == cy && x < y);
            });
            right.assign((size_t)nsplit + 1, 0.f);
            Box acc;
            acc.reset();
            for (int64_t i = np - 1; i >= kClusterTris; --i) {
                acc.grow(box[(size_t)srt[(size_t)i]]);
                if (i % kClusterTris == 0) right[(size_t)(i / kClusterTris)] = acc.area();
            }
            acc.reset();
            for (int64_t i = 0; i < np - 1; ++i) {
                acc.grow(box[(size_t)srt[(size_t)i]]);
                const int64_t at = i + 1;
                if (at % kClusterTris != 0) continue;
                const double cost = (double)acc.area() * (double)at +
                                    (double)right[(size_t)(at / kClusterTris)] * (double)(np - at);
                if (cost < best) {
                    best = cost;
                    best_axis = a;
                    best_at = at;
                }
            }
        }
        std::copy(sorted[best_axis].begin(), sorted[best_axis].end(), o.begin() + p.begin);
        const int64_t mid = p.begin + best_at;
        stack.push_back({mid, p.end});
        stack.push_back({p.begin, mid});
    }
}

}  // namespace pbg
