// pbg_rayhier.cu -- Accelerator "rayhierarchy": a hierarchy over the rays of
// each batch, rebuilt per call, traversed by the triangles.
//
// Reference: RayHieararchy (accelerators/rayhierarchy.cpp:375-1326) builds a
// quadtree over the batch's 2-D ray image -- leaves of chunkX x chunkY rays
// bounded by a 6-D box (origin AABB + direction AABB, bin/cl/rayhconstruct6DB.cl),
// parents by 2x2 merges (levelConstruct6DB.cl) -- and launches one thread per
// triangle that walks the tree with a global-memory stack
// (intersection6DB.cl:6-120), racing on tHit and repairing the races with
// extra passes (yetAnotherIntersection6DB.cl).
//
// Here:
//   build     rays ordered (pbg_rayorder.cu: the declared ray image in 2-D
//             Morton order, shadow batches along a 3-D Hilbert curve of their
//             origins, otherwise a 6-D Morton code) and gathered; a leaf is
//             32 consecutive rays (one warp builds it with shuffle
//             reductions); parents merge 4 children, up to the level the
//             descent is seeded at (no level above it is built).  A node is
//             bounded by an origin sphere (centre, radius), a direction cone
//             (unit axis, cos/sin of the half-angle) and the farthest reach
//             of its rays (max maxt*|d|).  A shadow batch whose origins and
//             validity repeat the previous batch's takes the kept order and
//             sorted origins at once; the comparison's answer is read with
//             the batch's closing status word and a batch whose origins moved
//             is traced again in a fresh order.
//   traverse  triangle records in clusters of 32 (SAH-style splits on whole
//             clusters, bvh_build.cpp), node test = "can any ray of the node
//             come within R of the triangle's or cluster's bounding sphere",
//             leaf test = the exact test per ray; the clusters walk the
//             levels level by level, seeded at the first level of at most
//             256 nodes; at the leaves'
//             parents a warp splits its cluster and tests the reaching
//             members against each leaf's rays directly; other split levels
//             group the (triangle, leaf) pairs by leaf first so a warp
//             loads a leaf's rays once for all its triangles.
//             Nearest hits merge through a 64-bit atomicMax on (t, index)
//             keys -- race-free by construction, no repair pass; a thread
//             reads a ray's current key first and filters with that t.
//             Nearest-hit batches take the final (cluster, leaves' parent)
//             pairs front to back (by distance from the parent's origin
//             ball) and cull with live reach bounds per leaf and parent.
//             Any-hit keeps one occlusion bit per ray (a 32-bit mask per
//             leaf) and skips leaves whose rays are all occluded.
#include <algorithm>
#include <functional>

#include "pbg_internal.h"
#include "pbg_count.cuh"
#include "pbg_tma.cuh"

namespace pbg {

int ray_sort(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
             const int32_t** perm, const uint32_t** sorted_keys, cudaStream_t st, int order);
int scan_counts(pbg_scene* s, uint32_t* a, int64_t m, cudaStream_t st);

constexpr int kLeafRays = 32;
constexpr int kFan = 4;
constexpr int kMaxLevels = 16;

struct __align__(16) RayNode {
    float4 a;  // origin sphere: centre.xyz, radius
    float4 b;  // cone axis.xyz, cos(half-angle)
    float4 c;  // sin(half-angle), reach = max maxt*|d|, count (int bits), unused
};

struct Levels {
    int64_t off[kMaxLevels];
    int64_t cnt[kMaxLevels];
    int nlev;
};

__device__ __forceinline__ float round_up_rel(float x) { return fmaf(fabsf(x), 0x1p-20f, x) + 0x1p-126f; }

// ---------------------------------------------------------------- build

// One warp per leaf of 32 sorted rays; the warp also gathers its rays into
// sorted order (so, sd) for the leaf tests.
// keep_o: the batch leaves from the same origins (bit for bit, mint
// included) in the same order as the previous one, whose sorted origins and
// leaf spheres are still in so / leaves: only the directions are gathered
// and only the cones rebuilt.
__global__ void leaf_build_kernel(const float4* __restrict__ ro, const float4* __restrict__ rd,
                                  const int32_t* __restrict__ perm, float4* __restrict__ so,
                                  float4* __restrict__ sd, const uint32_t* __restrict__ skeys, int64_t n,
                                  int64_t nleaf, RayNode* __restrict__ leaves, bool keep_o) {
    const int64_t leaf = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (leaf >= nleaf) return;
    const int64_t i = leaf * kLeafRays + lane;
    const bool ok = i < n && skeys[i] != 0xffffffffu;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
    if (ok) {  // invalid rays sort last and are never read back: not gathered
        const int32_t src = perm[i];
        d = rd[src];
        sd[i] = d;
        if (!keep_o) {
            o = ro[src];
            so[i] = o;
        }
    }
    const unsigned full = 0xffffffffu;
    const int count = __popc(__ballot_sync(full, ok));
    float lo[3] = {ok ? o.x : INFINITY, ok ? o.y : INFINITY, ok ? o.z : INFINITY};
    float hi[3] = {ok ? o.x : -INFINITY, ok ? o.y : -INFINITY, ok ? o.z : -INFINITY};
    const float len = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    const float il = len > 0.f ? 1.f / len : 0.f;
    float nx = d.x * il, ny = d.y * il, nz = d.z * il;
    float sx = ok ? nx : 0.f, sy = ok ? ny : 0.f, sz = ok ? nz : 0.f;
    float reach = ok ? d.w * len * (1.f + 0x1p-20f) : 0.f;
    if (ok && !(reach == reach)) reach = INFINITY;  // 0 * inf
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(full, lo[a], off));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(full, hi[a], off));
        }
        sx += __shfl_xor_sync(full, sx, off);
        sy += __shfl_xor_sync(full, sy, off);
        sz += __shfl_xor_sync(full, sz, off);
        reach = fmaxf(reach, __shfl_xor_sync(full, reach, off));
    }
    const float cx = 0.5f * (lo[0] + hi[0]), cy = 0.5f * (lo[1] + hi[1]), cz = 0.5f * (lo[2] + hi[2]);
    float dist = ok ? sqrtf((o.x - cx) * (o.x - cx) + (o.y - cy) * (o.y - cy) + (o.z - cz) * (o.z - cz)) : 0.f;
    const float sl = sqrtf(sx * sx + sy * sy + sz * sz);
    float ax = 0.f, ay = 0.f, az = 1.f;
    bool axis_ok = sl > 1e-3f * (float)(count > 0 ? count : 1);
    if (axis_ok) {
        ax = sx / sl;
        ay = sy / sl;
        az = sz / sl;
    }
    float cosv = ok ? (axis_ok ? ax * nx + ay * ny + az * nz : -1.f) : 2.f;
    if (ok && !(len > 0.f && isfinite(len))) cosv = -1.f;
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        dist = fmaxf(dist, __shfl_xor_sync(full, dist, off));
        cosv = fminf(cosv, __shfl_xor_sync(full, cosv, off));
    }
    if (lane == 0) {
        RayNode nd;
        if (count == 0) {
            nd.a = make_float4(0.f, 0.f, 0.f, 0.f);
            nd.b = make_float4(0.f, 0.f, 1.f, 1.f);
            nd.c = make_float4(0.f, 0.f, __int_as_float(0), 0.f);
        } else {
            // Margins: 2^-20 relative on the radius, 2^-18 on the cone cosine.
            const float ro_ = round_up_rel(dist);
            float c = fmaxf(cosv - 0x1p-18f, -1.f);
            if (c > 1.f) c = 1.f;
            const float s = fminf(sqrtf(fmaxf(0.f, 1.f - c * c)) + 0x1p-18f, 1.f);
            nd.a = keep_o ? leaves[leaf].a : make_float4(cx, cy, cz, ro_);
            nd.b = make_float4(ax, ay, az, c);
            nd.c = make_float4(s, reach, __int_as_float(count), 0.f);
        }
        leaves[leaf] = nd;
    }
}

// Parent j merges children kFan*j .. kFan*j+kFan-1.
__device__ __forceinline__ void build_parent(const RayNode* __restrict__ child, int64_t nchild,
                                             RayNode* __restrict__ parent, int64_t j) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float sx = 0.f, sy = 0.f, sz = 0.f, reach = 0.f;
    int count = 0;
    RayNode ch[kFan];
    int nk = 0;
    for (int k = 0; k < kFan; ++k) {
        const int64_t c = kFan * j + k;
        if (c >= nchild) break;
        ch[nk] = child[c];
        const int cc = __float_as_int(ch[nk].c.z);
        if (cc == 0) continue;
        const float4 a = ch[nk].a;
        lo[0] = fminf(lo[0], a.x - a.w); hi[0] = fmaxf(hi[0], a.x + a.w);
        lo[1] = fminf(lo[1], a.y - a.w); hi[1] = fmaxf(hi[1], a.y + a.w);
        lo[2] = fminf(lo[2], a.z - a.w); hi[2] = fmaxf(hi[2], a.z + a.w);
        sx += ch[nk].b.x * cc;
        sy += ch[nk].b.y * cc;
        sz += ch[nk].b.z * cc;
        reach = fmaxf(reach, ch[nk].c.y);
        count += cc;
        ++nk;
    }
    RayNode nd;
    if (count == 0) {
        nd.a = make_float4(0.f, 0.f, 0.f, 0.f);
        nd.b = make_float4(0.f, 0.f, 1.f, 1.f);
        nd.c = make_float4(0.f, 0.f, __int_as_float(0), 0.f);
        parent[j] = nd;
        return;
    }
    const float cx = 0.5f * (lo[0] + hi[0]), cy = 0.5f * (lo[1] + hi[1]), cz = 0.5f * (lo[2] + hi[2]);
    const float sl = sqrtf(sx * sx + sy * sy + sz * sz);
    const bool axis_ok = sl > 1e-3f * count;
    float ax = 0.f, ay = 0.f, az = 1.f;
    if (axis_ok) {
        ax = sx / sl;
        ay = sy / sl;
        az = sz / sl;
    }
    float r = 0.f, cmin = 1.f;
    for (int k = 0; k < nk; ++k) {
        const float4 a = ch[k].a;
        const float dx = a.x - cx, dy = a.y - cy, dz = a.z - cz;
        r = fmaxf(r, sqrtf(dx * dx + dy * dy + dz * dz) + a.w);
        // cos(angle(axis, child axis) + child half-angle)
        const float ca = axis_ok ? fminf(1.f, fmaxf(-1.f, ax * ch[k].b.x + ay * ch[k].b.y + az * ch[k].b.z)) : -1.f;
        const float sa = sqrtf(fmaxf(0.f, 1.f - ca * ca));
        const float cb = ch[k].b.w, sb = ch[k].c.x;
        // alpha + beta >= pi  <=>  cos(alpha) <= -cos(beta) (alpha, beta in [0, pi])
        const float csum = (ca <= -cb) ? -1.f : ca * cb - sa * sb;
        cmin = fminf(cmin, csum);
    }
    const float c = fmaxf(cmin - 0x1p-18f, -1.f);
    const float s = fminf(sqrtf(fmaxf(0.f, 1.f - c * c)) + 0x1p-18f, 1.f);
    nd.a = make_float4(cx, cy, cz, round_up_rel(r));
    nd.b = make_float4(ax, ay, az, c);
    nd.c = make_float4(s, reach, __int_as_float(count), 0.f);
    parent[j] = nd;
}

// Levels l0 + 1 .. l1 of the subtrees above groups of kFan^(l1 - l0) nodes
// of level l0: CTA g builds its subtree level by level (children written
// by the same CTA in the previous round), so five levels take one launch.
constexpr int kLevelsPerLaunch = 5;

__global__ void __launch_bounds__(256) level_build_multi_kernel(RayNode* __restrict__ nodes, Levels lv,
                                                                 int l0, int l1) {
    const int64_t span0 = 1ll << (2 * (l1 - l0));
    for (int l = l0 + 1; l <= l1; ++l) {
        const int64_t span = span0 >> (2 * (l - l0));
        const int64_t first = (int64_t)blockIdx.x * span;
        const int64_t last = min(first + span, lv.cnt[l]);
        for (int64_t j = first + threadIdx.x; j < last; j += blockDim.x)
            build_parent(nodes + lv.off[l - 1], lv.cnt[l - 1], nodes + lv.off[l], j);
        __syncthreads();
    }
}

// --------------------------------------------------------------- traverse

// Can a ray of node `nd` pass within reach of the sphere (c, r)?  r already
// holds the triangle's padding.  Conservative in float: every comparison
// carries a relative margin.
__device__ __forceinline__ bool node_hits_sphere(const RayNode& nd, float4 sph) {
    const float vx = sph.x - nd.a.x, vy = sph.y - nd.a.y, vz = sph.z - nd.a.z;
    const float dist2 = vx * vx + vy * vy + vz * vz;
    // Square roots by the hardware reciprocal square root (error a few ulp):
    // dist_lo / dist_hi bracket the distance by 2^-18, far inside the test's
    // own margins; 0 and inf give NaN, which keeps the pair.
    const float dist = dist2 * rsqrtf(dist2);
    const float dist_lo = dist * (1.f - 0x1p-18f), dist_hi = dist * (1.f + 0x1p-18f);
    // slop of pbrt's float test grows with the distance from the ray origin
    const float R = sph.w + nd.a.w + dist_hi * 0x1p-12f;
    if (!(dist_lo > R)) return true;  // overlapping (or NaN): keep
    if (dist_lo - R > nd.c.y * (1.f + 0x1p-18f)) return false;  // beyond every ray's maxt
    // With the sphere seen under half-angle beta (sin = R/dist, cos = q/dist)
    // and the cone's half-angle theta, the test is angle(axis, v) <= theta +
    // beta, i.e. axis.v >= dist cos(theta + beta) = cos(theta) q - sin(theta) R,
    // scaled by dist so that no division is needed.
    const float q2 = (dist_hi - R) * (dist_hi + R);  // > 0 here
    const float q = q2 * rsqrtf(q2);
    const float cth = nd.b.w, sth = nd.c.x;
    if (cth * dist <= -q) return true;  // cone half-angle + sphere angle >= pi
    const float dotv = vx * nd.b.x + vy * nd.b.y + vz * nd.b.z;
    return dotv >= cth * q - sth * R - 0x1p-16f * dist_hi;
}

// A (triangle record, node) pair that passed its node test.
struct Pair {
    int32_t tri;
    int32_t node;
};

// Appends up to kFan items per thread with one atomic per warp; items past
// the capacity are dropped and flagged (the host then reruns with smaller
// triangle groups).  Every lane of the warp must call it.
__device__ __forceinline__ void warp_append(const Pair* items, int k, Pair* q, uint32_t* count,
                                            uint32_t cap, int* status) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int incl = k;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(full, incl, off);
        if (lane >= off) incl += y;
    }
    const int total = __shfl_sync(full, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(count, (uint32_t)total);
    base = __shfl_sync(full, base, 31);
    const uint32_t start = base + (uint32_t)(incl - k);
    for (int j = 0; j < k; ++j) {
        const uint32_t pos = start + (uint32_t)j;
        if (pos < cap) q[pos] = items[j];
    }
    if (lane == 31 && total > 0 && base + (uint32_t)total > cap) atomicAdd(&status[kStatusOverflow], 1);
}

// Level-synchronous descent.  Pairs of level `lvl` (already tested) produce
// the pairs of their children that pass.  The descent is seeded at a level
// of at most kSeedNodes nodes: every (cluster or triangle in [t0, t1), node)
// pair there is tested directly, which replaces the launches of the nearly
// empty levels above it.
constexpr int64_t kSeedNodes = 256;

template <bool STATS>
__global__ void __launch_bounds__(256)
    rh_seed_kernel(const float4* __restrict__ spheres, int32_t t0, int32_t t1,
                   const RayNode* __restrict__ level_nodes, int64_t nnodes, Pair* __restrict__ out,
                   uint32_t* count, uint32_t cap, int* status, unsigned long long* wc) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t total = (int64_t)(t1 - t0) * nnodes;
    WorkCount c_;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < total; base += stride) {
        const int64_t i = base + threadIdx.x;
        Pair item[1];
        int k = 0;
        if (i < total) {
            const int64_t t = t0 + i / nnodes, node = i % nnodes;
            const RayNode nd = level_nodes[node];
            if (__float_as_int(nd.c.z) > 0) {
                if (STATS) c_.node++;
                if (node_hits_sphere(nd, spheres[t])) item[k++] = Pair{(int32_t)t, (int32_t)node};
            }
        }
        warp_append(item, k, out, count, cap, status);
    }
    if (STATS) c_.flush(wc);
}

template <bool STATS>
__global__ void __launch_bounds__(256)
    rh_expand_kernel(const float4* __restrict__ spheres, const RayNode* __restrict__ child_nodes,
                     int64_t nchild, const Pair* __restrict__ in, const uint32_t* __restrict__ in_count,
                     Pair* __restrict__ out, uint32_t* out_count, uint32_t cap, int* status,
                     unsigned long long* wc) {
    const uint32_t nin = min(*in_count, cap);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    WorkCount c_;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nin; base += stride) {
        const int64_t i = base + threadIdx.x;
        Pair item[kFan];
        int k = 0;
        if (i < nin) {
            const Pair p = in[i];
            const float4 sph = spheres[p.tri];
            const int64_t first = (int64_t)p.node * kFan;
            const int64_t last = min(first + kFan, nchild);
            for (int64_t c = first; c < last; ++c) {
                const RayNode nd = child_nodes[c];
                if (__float_as_int(nd.c.z) == 0) continue;
                if (STATS) c_.node++;
                if (node_hits_sphere(nd, sph)) item[k++] = Pair{p.tri, (int32_t)c};
            }
        }
        warp_append(item, k, out, out_count, cap, status);
    }
    if (STATS) c_.flush(wc);
}

// (cluster, node) pairs -> (triangle, node) pairs for the cluster's members
// in [t0, t1) whose own sphere passes the same node test: one warp per pair,
// lane j = member j.
template <bool STATS>
__global__ void __launch_bounds__(256)
    rh_split_kernel(const float4* __restrict__ spheres, int32_t t0, int32_t t1,
                    const RayNode* __restrict__ level_nodes, const Pair* __restrict__ in,
                    const uint32_t* __restrict__ in_count, Pair* __restrict__ out, uint32_t* out_count,
                    uint32_t cap, int* status, unsigned long long* wc) {
    const uint32_t nin = min(*in_count, cap);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    WorkCount c_;
    // every lane of a warp runs the same number of iterations (warp_append)
    for (int64_t p = warp; p < nin; p += nwarps) {
        const Pair pr = in[p];
        const int64_t t = (int64_t)pr.tri * kClusterTris + lane;
        Pair item[1];
        int k = 0;
        if (t >= t0 && t < t1) {
            const RayNode nd = level_nodes[pr.node];
            if (STATS) c_.node++;
            if (node_hits_sphere(nd, spheres[t])) item[k++] = Pair{(int32_t)t, pr.node};
        }
        warp_append(item, k, out, out_count, cap, status);
    }
    if (STATS) c_.flush(wc);
}

// The last two levels and the leaf tests in one pass, no pair queue: one
// warp per (cluster, leaves' parent) pair.  Lane j first stands for member
// triangle j (parent test, then each of the kFan leaves: a ballot gives the
// members that reach the leaf); then, leaf by leaf, lane k stands for ray k
// of the leaf and tests the reaching members one after another, their
// records staged in shared memory by the owning lanes.  A leaf's rays are
// loaded once per cluster that reaches it (from L2), instead of going
// through a written, counted, sorted and re-read list of (triangle, leaf)
// pairs.  Nearest: per-lane best key, atomicMax per leaf; any-hit: the
// leaf's occlusion bits are read first and set when a ray is blocked.
constexpr int kSplitTestMinBlocks = 5;  // CTAs per SM: measured best of 4-8 (5-7 equal, 5 spills least)
constexpr int kNearestMinBlocks = 4;     // nearest-hit variant, resident grid: best of 4-6

// Nearest-hit batches also keep a live reach bound per leaf and per leaves'
// parent: an upper bound on maxt x |d| over the node's rays, where each
// ray's maxt has shrunk to its best hit so far (hits are only replaced by
// nearer ones, or by the higher index at equal t, which the node test's
// strict comparison keeps).  A member whose sphere lies wholly beyond the
// bound cannot become any of the node's nearest hits, so it is culled like
// one beyond the rays' own maxt.  Stored as 0x7f800000 - bits(bound), so
// zeroed memory reads +inf and atomicMax lowers the bound.
__device__ __forceinline__ float live_reach(const uint32_t* b) {
    return __uint_as_float(0x7f800000u - __ldcg(b));
}
__device__ __forceinline__ void lower_reach(uint32_t* b, float x) {
    x = (x == x) ? fmaxf(x, 0.f) : INFINITY;  // NaN reads as unbounded
    atomicMax(b, 0x7f800000u - __float_as_uint(x));
}

template <bool ANY, bool STATS>
__global__ void __launch_bounds__(256, ANY ? kSplitTestMinBlocks : kNearestMinBlocks)
    rh_split_test_kernel(const float4* __restrict__ spheres, const TriRec* __restrict__ tris, int32_t t0,
                         int32_t t1, const RayNode* __restrict__ level1, const RayNode* __restrict__ leaves,
                         int64_t nleaf, const Pair* __restrict__ in, const uint32_t* __restrict__ in_count,
                         uint32_t cap, const float4* __restrict__ so, const float4* __restrict__ sd,
                         unsigned long long* __restrict__ keys, uint32_t* __restrict__ leafmask,
                         uint32_t* __restrict__ leaf_reach, uint32_t* __restrict__ parent_reach,
                         const int* __restrict__ status, unsigned long long* wc) {
    __shared__ float4 s_rec[8][kClusterTris * 3];  // this warp's member records (256 threads)
    if (status[kStatusOverflow] != 0) return;  // pairs were dropped upstream: this attempt is rerun
    const unsigned full = 0xffffffffu;
    float4* rec = s_rec[threadIdx.x >> 5];
    const uint32_t nin = min(*in_count, cap);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    WorkCount c_;
    for (int64_t p = warp; p < nin; p += nwarps) {
        const Pair pr = in[p];
        const int64_t t = (int64_t)pr.tri * kClusterTris + lane;
        bool pass = false;
        float4 sph = make_float4(0.f, 0.f, 0.f, 0.f);
        float parent_now = INFINITY;
        if (t >= t0 && t < t1) {
            sph = spheres[t];
            if (STATS) c_.node++;
            RayNode pn = level1[pr.node];
            if (!ANY) {
                pn.c.y = fminf(pn.c.y, live_reach(parent_reach + pr.node));
                parent_now = pn.c.y;
            }
            pass = node_hits_sphere(pn, sph);
        }
        if (!__any_sync(full, pass)) continue;
        __syncwarp();  // the previous pair's records are no longer read
        if (pass) {
            const TriRec own = tris[t];
            rec[3 * lane] = own.a;
            rec[3 * lane + 1] = own.b;
            rec[3 * lane + 2] = own.c;
        }
        __syncwarp();
        const int64_t first = (int64_t)pr.node * kFan;
        float parent_new = 0.f;  // max of the leaves' bounds after this pair
#pragma unroll 1
        for (int c = 0; c < kFan; ++c) {
            const int64_t leaf = first + c;
            if (leaf >= nleaf) break;
            RayNode nd = leaves[leaf];
            const int count = __float_as_int(nd.c.z);
            if (count == 0) continue;
            if (!ANY) nd.c.y = fminf(nd.c.y, live_reach(leaf_reach + leaf));
            bool reach = false;
            if (pass) {
                if (STATS) c_.node++;
                reach = node_hits_sphere(nd, sph);
            }
            unsigned m = __ballot_sync(full, reach);
            if (!m) {
                if (!ANY) parent_new = fmaxf(parent_new, nd.c.y);
                continue;
            }
            if (STATS && lane == 0) c_.leaf++;
            const int64_t r = leaf * kLeafRays + lane;
            bool active = lane < count;
            if (ANY && active) active = ((leafmask[leaf] >> lane) & 1u) == 0u;
            if (!__any_sync(full, active)) continue;
            float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
            float nd1 = 0.f, maxt = 0.f;
            unsigned long long best = 0ull, start = 0ull;
            if (active) {
                o = so[r];
                d = sd[r];
                nd1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
                maxt = d.w;
                if (!ANY) {
                    start = best = keys[r];
                    if (start != 0ull) maxt = fminf(maxt, key_t(start));
                }
            }
            bool hit = false;
            while (m) {
                const int j = __ffs(m) - 1;
                m &= m - 1;
                if (!active) continue;
                TriRec tr;
                tr.a = rec[3 * j];
                tr.b = rec[3 * j + 1];
                tr.c = rec[3 * j + 2];
                if (STATS) c_.filt++;
                if (!pbg_filter(tr, o, d, nd1, maxt)) continue;
                float tt, u1, u2;
                if (STATS) c_.exact++;
                if (!pbg_exact_rec(tr, o, d, maxt, &tt, &u1, &u2)) continue;
                if (STATS) c_.hit++;
                if (ANY) {
                    hit = true;
                    active = false;
                } else {
                    const unsigned long long k = hit_key(tt, __float_as_int(tr.c.w));
                    if (k > best) best = k;
                    maxt = tt;
                }
            }
            if (ANY) {
                if (hit) atomicOr(&leafmask[leaf], 1u << lane);
            } else {
                if (best > start) atomicMax(&keys[r], best);
                // the leaf's bound from its rays' maxt after this cluster
                // (2^-20 covers the rounding of |d|; lanes past count hold
                // no ray)
                const float len = sqrtf(fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)));
                float b = lane < count ? maxt * len * (1.f + 0x1p-20f) : 0.f;
                if (!(b == b)) b = INFINITY;
#pragma unroll
                for (int off = 16; off; off >>= 1) b = fmaxf(b, __shfl_xor_sync(full, b, off));
                if (lane == 0 && b < nd.c.y) lower_reach(leaf_reach + leaf, b);
                parent_new = fmaxf(parent_new, fminf(b, nd.c.y));
            }
        }
        if (!ANY && lane == 0 && parent_new < parent_now) lower_reach(parent_reach + pr.node, parent_new);
    }
    if (STATS) c_.flush(wc);
}

// Front-to-back order for the pairs of a nearest-hit batch: a counting sort
// of the (cluster, leaves' parent) pairs on the distance from the parent's
// origin ball to the cluster's sphere, so that the leaf tests, which take
// the pairs in queue order over time, meet the near clusters first and
// their hits lower the live reach bounds before the far clusters arrive.
// Buckets: the top bits of the float distance, 64 per octave.  The order
// only changes how much is culled, never a result.
constexpr int kOrderBuckets = 16384;

__device__ __forceinline__ uint32_t pair_bucket(float4 c, float4 ball) {
    const float dx = c.x - ball.x, dy = c.y - ball.y, dz = c.z - ball.z;
    float dist = sqrtf(dx * dx + dy * dy + dz * dz) - c.w - ball.w;
    if (!(dist > 0.f)) dist = 0.f;  // overlapping, or NaN
    return min(__float_as_uint(dist) >> 17, (uint32_t)kOrderBuckets - 1u);
}

__global__ void __launch_bounds__(256)
    rh_order_count_kernel(const float4* __restrict__ csph, const RayNode* __restrict__ level1,
                          const Pair* __restrict__ in, const uint32_t* __restrict__ in_count, uint32_t cap,
                          uint32_t* __restrict__ hist, const int* __restrict__ status) {
    if (status[kStatusOverflow] != 0) return;  // this attempt is rerun
    const uint32_t nin = min(*in_count, cap);
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nin; base += stride) {
        const int64_t i = base + threadIdx.x;
        const bool ok = i < nin;
        uint32_t key = (uint32_t)kOrderBuckets;
        if (ok) {
            const Pair pr = in[i];
            key = pair_bucket(csph[pr.tri], level1[pr.node].a);
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        if (ok && lane == __ffs(peers) - 1) atomicAdd(&hist[key], (uint32_t)__popc(peers));
    }
}

__global__ void __launch_bounds__(256)
    rh_order_scatter_kernel(const float4* __restrict__ csph, const RayNode* __restrict__ level1,
                            const Pair* __restrict__ in, const uint32_t* __restrict__ in_count, uint32_t cap,
                            uint32_t* __restrict__ cursor, Pair* __restrict__ out,
                            const int* __restrict__ status) {
    if (status[kStatusOverflow] != 0) return;
    const uint32_t nin = min(*in_count, cap);
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nin; base += stride) {
        const int64_t i = base + threadIdx.x;
        const bool ok = i < nin;
        Pair pr = Pair{0, 0};
        uint32_t key = (uint32_t)kOrderBuckets;
        if (ok) {
            pr = in[i];
            key = pair_bucket(csph[pr.tri], level1[pr.node].a);
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        uint32_t first = 0;
        if (ok && lane == leader) first = atomicAdd(&cursor[key], (uint32_t)__popc(peers));
        first = __shfl_sync(0xffffffffu, first, leader);
        const uint64_t dst = (uint64_t)first + __popc(peers & lt);
        if (ok && dst < nin) out[dst] = pr;
    }
}

// The final pairs grouped by leaf (a counting sort: count with ranks, scan,
// scatter), so that a leaf's 32 rays are loaded once for all the triangles
// that reach it instead of once per pair.
__global__ void rh_leaf_count_kernel(const Pair* __restrict__ in, const uint32_t* __restrict__ in_count,
                                     uint32_t cap, uint32_t* __restrict__ leafcnt,
                                     uint32_t* __restrict__ rank) {
    const uint32_t nin = min(*in_count, cap);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nin; i += stride)
        rank[i] = atomicAdd(&leafcnt[in[i].node], 1u);
}

// After a queue overflow (pairs dropped; the host reruns the batch with more
// triangle groups) the counts and ranks no longer describe the queue, so the
// sort and the leaf tests of that attempt do nothing.
__global__ void rh_leaf_scatter_kernel(const Pair* __restrict__ in, const uint32_t* __restrict__ in_count,
                                       uint32_t cap, const uint32_t* __restrict__ leafoff,
                                       const uint32_t* __restrict__ rank, Pair* __restrict__ out,
                                       const int* __restrict__ status) {
    if (status[kStatusOverflow] != 0) return;
    const uint32_t nin = min(*in_count, cap);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nin; i += stride) {
        const Pair p = in[i];
        const uint64_t dst = (uint64_t)leafoff[p.node] + rank[i];
        if (dst < nin) out[dst] = p;
    }
}

constexpr int kLeafChunk = 64;
constexpr int kLeafWarps = 8;  // warps per CTA of the leaf kernel

// One warp per chunk of kLeafChunk leaf-sorted pairs.  The chunk's pairs and
// triangle records are first staged in shared memory by the whole warp (so
// the loads overlap), then lane k tests ray k of the current leaf (loaded
// when the leaf changes) against each record.  Nearest: each lane keeps its
// best key and shrinks its maxt as it finds hits, merging with atomicMax
// when the leaf changes.  Any-hit: an occluded lane stops and sets its bit
// on leaving.
template <bool ANY, bool STATS>
__global__ void __launch_bounds__(32 * kLeafWarps)
    rh_leaf_sorted_kernel(const TriRec* __restrict__ tris, const RayNode* __restrict__ leaves,
                          const Pair* __restrict__ in, const uint32_t* __restrict__ in_count,
                          uint32_t cap, const float4* __restrict__ so, const float4* __restrict__ sd,
                          unsigned long long* __restrict__ keys, uint32_t* __restrict__ leafmask,
                          const int* __restrict__ status, unsigned long long* wc) {
    __shared__ float4 s_tri[kLeafWarps][kLeafChunk * 3];
    __shared__ Pair s_pair[kLeafWarps][kLeafChunk];
    if (status[kStatusOverflow] != 0) return;  // this attempt is rerun
    const uint32_t nin = min(*in_count, cap);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float4* t4 = reinterpret_cast<const float4*>(tris);
    Pair* sp = s_pair[wib];
    float4* st4 = s_tri[wib];
    WorkCount c_;
    for (int64_t c0 = warp * kLeafChunk; c0 < nin; c0 += nwarps * kLeafChunk) {
        const int cnt = (int)min((int64_t)kLeafChunk, (int64_t)nin - c0);
        for (int j = lane; j < cnt; j += 32) sp[j] = in[c0 + j];
        __syncwarp();
        for (int j = lane; j < 3 * cnt; j += 32) st4[j] = t4[(int64_t)sp[j / 3].tri * 3 + j % 3];
        __syncwarp();
        int32_t leaf = -1;
        bool active = false, hit = false;
        int64_t r = 0;
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
        float nd1 = 0.f, maxt = 0.f;
        unsigned long long best = 0ull, start = 0ull;
        for (int p = 0; p < cnt; ++p) {
            const Pair pr = sp[p];
            if (pr.node != leaf) {
                if (ANY) {
                    if (hit) atomicOr(&leafmask[leaf], 1u << lane);
                } else if (best > start) {
                    atomicMax(&keys[r], best);
                }
                leaf = pr.node;
                if (STATS && lane == 0) c_.leaf++;
                const int count = __float_as_int(leaves[leaf].c.z);
                r = (int64_t)leaf * kLeafRays + lane;
                active = lane < count;
                if (ANY && active) active = ((leafmask[leaf] >> lane) & 1u) == 0u;
                hit = false;
                if (active) {
                    o = so[r];
                    d = sd[r];
                    nd1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
                    maxt = d.w;
                    if (!ANY) {
                        start = best = keys[r];
                        if (start != 0ull) maxt = fminf(maxt, key_t(start));
                    }
                } else {
                    start = best = 0ull;
                }
            }
            if (!active) continue;
            TriRec tr;
            tr.a = st4[3 * p];
            tr.b = st4[3 * p + 1];
            tr.c = st4[3 * p + 2];
            if (STATS) c_.filt++;
            if (!pbg_filter(tr, o, d, nd1, maxt)) continue;
            float tt, u1, u2;
            if (STATS) c_.exact++;
            if (!pbg_exact_rec(tr, o, d, maxt, &tt, &u1, &u2)) continue;
            if (STATS) c_.hit++;
            if (ANY) {
                hit = true;
                active = false;
            } else {
                const unsigned long long k = hit_key(tt, __float_as_int(tr.c.w));
                if (k > best) best = k;
                maxt = tt;
            }
        }
        if (leaf >= 0) {
            if (ANY) {
                if (hit) atomicOr(&leafmask[leaf], 1u << lane);
            } else if (best > start) {
                atomicMax(&keys[r], best);
            }
        }
        __syncwarp();  // the next chunk overwrites this warp's staging
    }
    if (STATS) c_.flush(wc);
}

// Sorted-order results back to the caller's order.
__global__ void rh_finalize_nearest(const TriRec* __restrict__ tris, const int32_t* __restrict__ pos,
                                    const float4* __restrict__ so, const float4* __restrict__ sd,
                                    const int32_t* __restrict__ perm,
                                    const unsigned long long* __restrict__ keys, int64_t n,
                                    int32_t* prim, float* t, float* b1, float* b2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t ray = perm[i];
    const unsigned long long k = keys[i];
    int32_t p = -1;
    float tt = 0.f, u1 = 0.f, u2 = 0.f;
    if (k != 0ull) {
        p = key_prim(k);
        const float4 o = so[i], d = sd[i];
        if (!pbg_exact_rec(tris[pos[p]], o, d, d.w, &tt, &u1, &u2)) {
            p = -1;
            tt = u1 = u2 = 0.f;
        }
    }
    prim[ray] = p;
    t[ray] = tt;
    b1[ray] = u1;
    b2[ray] = u2;
}

__global__ void rh_finalize_occluded(const int32_t* __restrict__ perm,
                                     const uint32_t* __restrict__ leafmask, int64_t n,
                                     uint8_t* occ) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    occ[perm[i]] = (leafmask[i / kLeafRays] >> (i % kLeafRays)) & 1u;
}

// ------------------------------------------------------------------ host

// The levels the traversal reads: clusters split into triangles at level
// `split`, and the descent is seeded at `seed`, the lowest level of at most
// kSeedNodes (tune.rh_seed) nodes not below max(split, 1).  No level above the seed is
// read, so the build stops there.
struct Descent {
    int split, seed;
};
static Descent descent_levels(const pbg_scene* s, const Levels& lv, bool any) {
    const int top = lv.nlev - 1;
    // levels walked by 32-triangle clusters before they split into triangles
    // (default: down to the leaves' parents, the fastest split on the
    // terrain direct-lighting frame)
    int kcl = s->params.rh_cluster_levels;
    if (kcl == 0) kcl = std::max(1, top - 1);
    if (kcl < 0 || s->clusters.ptr == nullptr) kcl = 0;
    Descent d;
    d.split = std::max(0, top - kcl);
    d.seed = top;
    const int64_t seed_nodes = s->tune.rh_seed[any] > 0 ? s->tune.rh_seed[any] : kSeedNodes;
    while (d.seed > std::max(d.split, 1) && lv.cnt[d.seed - 1] <= seed_nodes) --d.seed;
    return d;
}

static int rh_build(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                    const int32_t** perm, float4** so, float4** sd, Levels* lv, int order,
                    cudaStream_t st) {
    Work& w = s->work;
    const uint32_t* skeys = nullptr;
    const bool had_origins = w.sorted_origins_ok;
    w.sorted_origins_ok = false;  // set again once this hierarchy build has written them
    const void* before[2] = {w.ray_o2.ptr, w.nodes.ptr};
    int rc = ray_sort(s, o, d, valid, n, perm, &skeys, st, order);
    if (rc) return rc;
    if ((rc = ensure(w.ray_o2, (size_t)n * sizeof(float4))) ||
        (rc = ensure(w.ray_d2, (size_t)n * sizeof(float4))))
        return rc;
    *so = (float4*)w.ray_o2.ptr;
    *sd = (float4*)w.ray_d2.ptr;
    // levels: leaves of 32 rays, parents of 4 children, up to one root
    int64_t cnt = (n + kLeafRays - 1) / kLeafRays, total = 0;
    lv->nlev = 0;
    for (;;) {
        lv->off[lv->nlev] = total;
        lv->cnt[lv->nlev] = cnt;
        total += cnt;
        lv->nlev++;
        if (cnt <= 1 || lv->nlev == kMaxLevels) break;
        cnt = (cnt + kFan - 1) / kFan;
    }
    if ((rc = ensure(w.nodes, (size_t)total * sizeof(RayNode)))) return rc;
    RayNode* nodes = (RayNode*)w.nodes.ptr;
    const int64_t nleaf = lv->cnt[0];
    // the previous batch's sorted origins and leaf spheres still apply when
    // its order was reused and neither buffer moved
    const bool keep_o = order == kOrderOrigin && w.origin_reused && had_origins &&
                        before[0] == w.ray_o2.ptr && before[1] == w.nodes.ptr;
    prof_begin(s, st);
    leaf_build_kernel<<<(unsigned)((nleaf * 32 + 255) / 256), 256, 0, st>>>(o, d, *perm, *so, *sd, skeys,
                                                                            n, nleaf, nodes, keep_o);
    prof_end(s, st, kStageBuild, 1);
    // the levels above are never read (any-hit batches are the origin-ordered ones)
    const int built = descent_levels(s, *lv, order == kOrderOrigin).seed;
    for (int l0 = 0; l0 < built; l0 += kLevelsPerLaunch) {
        const int l1 = std::min(l0 + kLevelsPerLaunch, built);
        const int64_t group = 1ll << (2 * (l1 - l0));
        prof_begin(s, st);
        level_build_multi_kernel<<<(unsigned)((lv->cnt[l0] + group - 1) / group), 256, 0, st>>>(nodes, *lv,
                                                                                               l0, l1);
        prof_end(s, st, kStageBuild, 1);
    }
    PBG_CUDA(cudaGetLastError());
    w.sorted_origins_ok = order == kOrderOrigin;
    return PBG_OK;
}

// Pairs per queue buffer: 2^25 (256 MB) unless the scene's parameters set
// another capacity; a batch that overflows it reruns with the triangles split
// into more groups.
constexpr uint32_t kQueueCap = 1u << 25;
constexpr uint32_t kQueueCapMin = 4096;

static uint32_t queue_capacity(const pbg_scene* s) {
    const int32_t q = s->params.rh_queue_pairs;
    return q > 0 ? std::max<uint32_t>((uint32_t)q, kQueueCapMin) : kQueueCap;
}

template <bool ANY>
static int rh_traverse(pbg_scene* s, const Levels& lv, const float4* so, const float4* sd,
                       unsigned long long* keys, uint32_t* mask, cudaStream_t st, int* moved,
                       const std::function<int()>& tail) {
    Work& w = s->work;
    int rc;
    const int64_t nleaf = lv.cnt[0];
    const uint32_t cap = queue_capacity(s);
    if ((rc = ensure(w.queue_a, (size_t)cap * sizeof(Pair))) ||
        (rc = ensure(w.queue_b, (size_t)cap * sizeof(Pair))) ||
        (rc = ensure(w.pair_rank, (size_t)cap * sizeof(uint32_t))) ||
        (rc = ensure(w.leafcnt, (size_t)nleaf * sizeof(uint32_t))) ||
        (rc = ensure(w.qcount, 64 * sizeof(uint32_t))))
        return rc;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    // grid-stride kernels: 32 CTAs per SM measured best of 4, 8, 16, 32 on
    // the terrain frame (tune.rh_grid)
    const unsigned grid = (unsigned)(sms * (s->tune.rh_grid[ANY] > 0 ? s->tune.rh_grid[ANY] : 32));
    const bool stats = s->prof.level >= 2;
    unsigned long long* wc = (unsigned long long*)s->workc.ptr;
    int* status = (int*)s->err.ptr;
    const RayNode* nodes = (const RayNode*)w.nodes.ptr;
    uint32_t* counts = (uint32_t*)w.qcount.ptr;
    static_assert(2 * kMaxLevels <= 64, "pair counters");
    int groups = s->rh_groups > 0 ? s->rh_groups : 1;
    const int top = lv.nlev - 1;
    const Descent dsc = descent_levels(s, lv, ANY);
    const int split = dsc.split;
    const int kcl = top - split;  // levels walked by clusters (0: none)
    const float4* tsph = (const float4*)s->spheres.ptr;
    const float4* csph = (const float4*)s->clusters.ptr;
    uint32_t *leaf_reach = nullptr, *parent_reach = nullptr, *order_hist = nullptr;
    if (!ANY && lv.nlev > 1) {  // live reach bounds, +inf to start (zeroed)
        const size_t nb = (size_t)(lv.cnt[0] + lv.cnt[1]);
        if ((rc = ensure(w.reach, (nb + kOrderBuckets) * sizeof(uint32_t)))) return rc;
        leaf_reach = (uint32_t*)w.reach.ptr;
        parent_reach = leaf_reach + lv.cnt[0];
        order_hist = parent_reach + lv.cnt[1];
        PBG_CUDA(cudaMemsetAsync(leaf_reach, 0, nb * sizeof(uint32_t), st));
    }
    for (int attempt = 0; attempt < 8; ++attempt) {
        PBG_CUDA(cudaMemsetAsync(status + kStatusOverflow, 0, sizeof(int), st));
        // group boundaries on cluster boundaries
        const int64_t per = ((s->ntri + groups - 1) / groups + kClusterTris - 1) / kClusterTris * kClusterTris;
        for (int g = 0; g < groups; ++g) {
            const int32_t t0 = (int32_t)std::min<int64_t>(s->ntri, g * per),
                          t1 = (int32_t)std::min<int64_t>(s->ntri, (g + 1) * per);
            if (t0 >= t1) break;
            PBG_CUDA(cudaMemsetAsync(counts, 0, 64 * sizeof(uint32_t), st));
            Pair* qa = (Pair*)w.queue_a.ptr;
            Pair* qb = (Pair*)w.queue_b.ptr;
            prof_begin(s, st);
            int nl = 1;  // kernels launched below (scan_counts counts its own)
            // pairs of level l count in counts[l] (clusters: counts[kMaxLevels + l])
            const bool cl = kcl > 0;
            const float4* seed_sph = cl ? csph : tsph;
            const int32_t s0 = cl ? t0 / kClusterTris : t0;
            const int32_t s1 = cl ? (int32_t)((t1 + kClusterTris - 1) / kClusterTris) : t1;
            uint32_t* cnt_of[kMaxLevels];
            for (int l = 0; l < kMaxLevels; ++l) cnt_of[l] = &counts[(cl && l >= split) ? kMaxLevels + l : l];
            // seed level: the lowest with at most kSeedNodes nodes, not below
            // the level where clusters split
            const int ls = dsc.seed;
            const int64_t seed_grid = std::min<int64_t>(
                grid, ((int64_t)(s1 - s0) * lv.cnt[ls] + 255) / 256);
            if (stats)
                rh_seed_kernel<true><<<(unsigned)seed_grid, 256, 0, st>>>(
                    seed_sph, s0, s1, nodes + lv.off[ls], lv.cnt[ls], qa, cnt_of[ls], cap, status, wc);
            else
                rh_seed_kernel<false><<<(unsigned)seed_grid, 256, 0, st>>>(
                    seed_sph, s0, s1, nodes + lv.off[ls], lv.cnt[ls], qa, cnt_of[ls], cap, status,
                    nullptr);
            uint32_t* leafcnt = (uint32_t*)w.leafcnt.ptr;
            uint32_t* rank = (uint32_t*)w.pair_rank.ptr;
            if (!(cl && split == 1))  // the leaf-pair counting sort runs
                PBG_CUDA(cudaMemsetAsync(leafcnt, 0, (size_t)nleaf * sizeof(uint32_t), st));
            bool fused = false;
            for (int l = ls; l >= 0; --l) {
                if (cl && l == 1 && split == 1) {  // clusters straight into the leaf tests
                    unsigned tgrid = grid * 2;
                    if (order_hist) {  // nearest: front-to-back pairs, taken in order
                        PBG_CUDA(cudaMemsetAsync(order_hist, 0, kOrderBuckets * sizeof(uint32_t), st));
                        rh_order_count_kernel<<<grid, 256, 0, st>>>(csph, nodes + lv.off[1], qa, cnt_of[1],
                                                                    cap, order_hist, status);
                        if ((rc = scan_counts(s, order_hist, kOrderBuckets, st))) return rc;
                        rh_order_scatter_kernel<<<grid, 256, 0, st>>>(csph, nodes + lv.off[1], qa,
                                                                      cnt_of[1], cap, order_hist, qb,
                                                                      status);
                        Pair* tq = qa;
                        qa = qb;
                        qb = tq;
                        tgrid = (unsigned)(sms * kNearestMinBlocks);  // resident CTAs only
                        nl += 2;
                    }
                    if (stats)
                        rh_split_test_kernel<ANY, true><<<tgrid, 256, 0, st>>>(
                            tsph, (const TriRec*)s->tris.ptr, t0, t1, nodes + lv.off[1], nodes + lv.off[0],
                            lv.cnt[0], qa, cnt_of[1], cap, so, sd, keys, mask, leaf_reach,
                            parent_reach, status, wc);
                    else
                        rh_split_test_kernel<ANY, false><<<tgrid, 256, 0, st>>>(
                            tsph, (const TriRec*)s->tris.ptr, t0, t1, nodes + lv.off[1], nodes + lv.off[0],
                            lv.cnt[0], qa, cnt_of[1], cap, so, sd, keys, mask, leaf_reach,
                            parent_reach, status, nullptr);
                    fused = true;
                    ++nl;
                    break;
                }
                if (cl && l == split) {  // clusters -> triangles, same level
                    if (stats)
                        rh_split_kernel<true><<<grid * 2, 256, 0, st>>>(
                            tsph, t0, t1, nodes + lv.off[l], qa, cnt_of[l], qb, &counts[l], cap,
                            status, wc);
                    else
                        rh_split_kernel<false><<<grid * 2, 256, 0, st>>>(
                            tsph, t0, t1, nodes + lv.off[l], qa, cnt_of[l], qb, &counts[l], cap,
                            status, nullptr);
                    Pair* tq = qa;
                    qa = qb;
                    qb = tq;
                    cnt_of[l] = &counts[l];
                    ++nl;
                }
                if (l == 0) break;
                const float4* sph = (cl && l > split) ? csph : tsph;
                if (stats)
                    rh_expand_kernel<true><<<grid, 256, 0, st>>>(
                        sph, nodes + lv.off[l - 1], lv.cnt[l - 1], qa, cnt_of[l], qb, cnt_of[l - 1],
                        cap, status, wc);
                else
                    rh_expand_kernel<false><<<grid, 256, 0, st>>>(
                        sph, nodes + lv.off[l - 1], lv.cnt[l - 1], qa, cnt_of[l], qb, cnt_of[l - 1],
                        cap, status, nullptr);
                Pair* tq = qa;
                qa = qb;
                qb = tq;
                ++nl;
            }
            // group the leaf pairs by leaf (qa -> qb), then the leaf tests
            if (!fused) {
                rh_leaf_count_kernel<<<grid, 256, 0, st>>>(qa, &counts[0], cap, leafcnt, rank);
                if ((rc = scan_counts(s, leafcnt, nleaf, st))) return rc;
                rh_leaf_scatter_kernel<<<grid, 256, 0, st>>>(qa, &counts[0], cap, leafcnt, rank, qb,
                                                             status);
                if (stats)
                    rh_leaf_sorted_kernel<ANY, true><<<grid * 2, 32 * kLeafWarps, 0, st>>>(
                        (const TriRec*)s->tris.ptr, nodes, qb, &counts[0], cap, so, sd, keys, mask,
                        status, wc);
                else
                    rh_leaf_sorted_kernel<ANY, false><<<grid * 2, 32 * kLeafWarps, 0, st>>>(
                        (const TriRec*)s->tris.ptr, nodes, qb, &counts[0], cap, so, sd, keys, mask,
                        status, nullptr);
                nl += 3;
            }
            prof_end(s, st, kStageTraverse, nl);
            PBG_CUDA(cudaGetLastError());
        }
        // One status read per call: a dropped pair would lose hits.  With
        // *moved, the word after it too: the batch's origins differ from
        // the kept order it was traced in, and the caller traces it again.
        // The caller's tail (the finalize kernel) is enqueued behind the
        // publication, so the GPU runs it while the host waits; an attempt
        // that is rerun enqueues it again.
        int seq = 0;
        if ((rc = publish_device_words(s, status + kStatusOverflow, moved ? 2 : 1, &seq, st))) return rc;
        if ((rc = tail())) return rc;
        int h[2] = {0, 0};
        if ((rc = wait_device_words(s, seq, moved ? 2 : 1, h, st))) return rc;
        if (moved && h[1] != 0) {
            *moved = 1;
            return PBG_OK;
        }
        if (h[0] == 0) return PBG_OK;
        groups *= 4;  // rerun: atomicMax / atomicOr merges make a rerun idempotent
        s->rh_groups = groups;
        s->counters.queue_reruns++;
    }
    set_last_error("rayhierarchy: pair queues overflowed at every triangle grouping");
    return PBG_ERR_INTERNAL;
}

int rh_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
               int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    // A nearest-hit batch yields new hit points: the origin order kept for
    // the shadow batches that leave from the previous ones is dropped, so
    // only shadow batches between two nearest-hit batches share a sort.
    s->work.origin_sort_n = -1;
    s->alt.origin_sort_n = -1;
    const int32_t* perm;
    float4 *so, *sd;
    Levels lv;
    int rc = rh_build(s, o, d, valid, n, &perm, &so, &sd, &lv, kOrderDefault, st);
    if (rc) return rc;
    Work& w = s->work;
    if ((rc = ensure(w.keys, (size_t)n * 8))) return rc;
    unsigned long long* keys = (unsigned long long*)w.keys.ptr;
    PBG_CUDA(cudaMemsetAsync(keys, 0, (size_t)n * 8, st));
    const std::function<int()> finalize = [&]() -> int {
        prof_begin(s, st);
        rh_finalize_nearest<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
            (const TriRec*)s->tris.ptr, (const int32_t*)s->tri_pos.ptr, so, sd, perm, keys, n, prim, t, b1,
            b2);
        prof_end(s, st, kStageOther, 1);
        PBG_CUDA(cudaGetLastError());
        return PBG_OK;
    };
    if (s->ntri > 0) return rh_traverse<false>(s, lv, so, sd, keys, nullptr, st, nullptr, finalize);
    return finalize();
}

int rh_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                uint8_t* occ, cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    // Two attempts at most: one in the kept origin order, taken before the
    // comparison's answer, and, when the origins moved, one in a fresh order
    // (the kept order is dropped, so that attempt cannot speculate).
    for (int attempt = 0; attempt < 2; ++attempt) {
        const int32_t* perm;
        float4 *so, *sd;
        Levels lv;
        int rc = rh_build(s, o, d, valid, n, &perm, &so, &sd, &lv, kOrderOrigin, st);
        if (rc) return rc;
        Work& w = s->work;
        const bool speculative = w.origin_speculative;
        const int64_t nleaf = lv.cnt[0];
        if ((rc = ensure(w.leafmask, (size_t)nleaf * 4))) return rc;
        uint32_t* mask = (uint32_t*)w.leafmask.ptr;
        PBG_CUDA(cudaMemsetAsync(mask, 0, (size_t)nleaf * 4, st));
        const std::function<int()> finalize = [&]() -> int {
            prof_begin(s, st);
            rh_finalize_occluded<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(perm, mask, n, occ);
            prof_end(s, st, kStageOther, 1);
            PBG_CUDA(cudaGetLastError());
            return PBG_OK;
        };
        int moved = 0;
        if (s->ntri > 0) {
            // the finalize runs behind the status publication; a moved
            // batch's answers are overwritten by the next attempt's
            rc = rh_traverse<true>(s, lv, so, sd, nullptr, mask, st, speculative ? &moved : nullptr, finalize);
            if (rc) return rc;
        } else {
            if ((rc = finalize())) return rc;
            if (speculative &&
                (rc = read_device_words(s, (const int*)s->err.ptr + kStatusOriginMoved, 1, &moved, st)))
                return rc;
        }
        if (moved) {
            w.origin_sort_n = -1;
            w.origin_reused = w.origin_speculative = false;
            s->counters.origin_reruns++;
            continue;
        }
        if (speculative) s->counters.origin_reuses++;
        return PBG_OK;
    }
    set_last_error("rayhierarchy: the origin order changed under a fresh sort");
    return PBG_ERR_INTERNAL;
}

}  // namespace pbg
