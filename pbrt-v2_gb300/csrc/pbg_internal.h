// pbg_internal.h -- host-side state shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pbrt_gb300.h"
#include "pbg_exact.cuh"

namespace pbg {

struct Learner;
struct RenderBuffers;

// Two-wide BVH node (64 bytes): both children's boxes, so one node fetch
// decides both children.  A child index >= 0 is an inner node; a negative
// index ~start is a leaf holding triangles [start, start + count).
struct __align__(16) BvhNode {
    float4 n0;  // c0.lo.x c0.hi.x c0.lo.y c0.hi.y
    float4 n1;  // c1.lo.x c1.hi.x c1.lo.y c1.hi.y
    float4 n2;  // c0.lo.z c0.hi.z c1.lo.z c1.hi.z
    int4 n3;    // child0, child1, count0, count1
};

// Event pairs around launches, summed per stage when counters are read.
struct Profiler {
    bool on = false;
    int level = 0;  // 2: count traversal work
    struct Rec {
        cudaEvent_t a, b;
        int stage;
    };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
};

struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// Error-reporting helpers: every entry point returns a pbg status and keeps
// the text of the last failure in a thread-local string.
void set_last_error(const std::string& msg);
int cuda_status(cudaError_t e, const char* what);

#define PBG_CUDA(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_status(e_, #call); \
    } while (0)

int ensure(DeviceBuffer& b, size_t bytes);
void release(DeviceBuffer& b);

// Host-built SAH BVH over the triangles (bvh_build.cpp).  order[i] = the
// original index of the i-th triangle in leaf order.
struct HostBvh {
    std::vector<BvhNode> nodes;
    std::vector<int32_t> order;
    int max_depth = 0;
    int32_t unculled = 0;  // order[0, unculled): degenerate, outside the tree
};
bool triangle_degenerate(const float* v9);
void build_bvh(const float* tri9, int64_t ntri, int max_leaf, HostBvh* out);

// Ray orders of ray_sort(): the declared ray image if any, else 6-D Morton;
// or the origins along a 3-D Hilbert curve.
enum { kOrderDefault = 0, kOrderOrigin = 1 };

// Records per rayhierarchy triangle cluster (one warp splits a cluster).
constexpr int kClusterTris = 32;

// Launch-shape settings that change no result, chosen by pbg_autotune (the
// defaults are the shapes measured best on the benchmark scenes).
struct Tunables {
    int naive_ctas = 4;      // naive: CTAs per SM the triangle splits aim for
    // rayhierarchy [any-hit]: nodes of the level the descent starts at (at
    // most), CTAs per SM of the grid-stride kernels
    int rh_seed[2] = {256, 256};
    int rh_grid[2] = {32, 32};
    int bvh_walk[2][2] = {{0, 0}, {0, 0}};  // ray-bvh [any-hit][incoherent]: 0 automatic, else pbg_params.walk's 1-6
};

// Per-batch device scratch owned by a scene.
struct Work {
    DeviceBuffer ray_o, ray_d, ray_o2, ray_d2, valid, prim, t, b1, b2, occ, keys, stage, perm,
        perm_tmp, mkeys, mkeys_tmp, hist, nodes, leafmask, counters, geo, queue_a, queue_b,
        qcount, scan_sums, pair_rank, leafcnt, origin_cache, osort_keys, osort_perm, reach, origin_valid;
    int64_t cap = 0;
    int64_t origin_sort_n = -1;      // rays of the cached origin sort (-1 = none)
    bool origin_reused = false;      // the last origin-ordered sort reused the kept order
    bool origin_speculative = false; // ... before the comparison's answer was read
    bool sorted_origins_ok = false;  // ray_o2 and the leaves hold the last origin-ordered
                                     // build's sorted origins and leaf spheres
};
void release_work(Work& w);

}  // namespace pbg

struct pbg_scene {
    int device = 0;
    int32_t accel = 0;
    pbg_params params{};
    int64_t ntri = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t io_stream = nullptr;          // host-link copies of two-half calls
    cudaEvent_t io_events[8] = {};
    pbg::DeviceBuffer tris;    // TriRec[ntri], in traversal order (c.w = original index)
    pbg::DeviceBuffer tri9;    // original vertices, float[9*ntri]
    pbg::DeviceBuffer uv6;     // optional per-triangle uvs, float[6*ntri]
    pbg::DeviceBuffer bvh;     // BvhNode[] (ray-bvh)
    pbg::DeviceBuffer wide;    // WideNode[] (ray-bvh walks 5 and 6, built on their first batch)
    pbg::DeviceBuffer tris_wide; // TriRec[ntri] in the wide tree's leaf order
    int64_t wide_nodes = 0;
    std::vector<int32_t> bvh_levels;  // device-built tree: (first node, nodes) per level, root first
    int wide_state = 0;        // 0 not built yet, 1 built, -1 the tree does not fit the wide format
    pbg::DeviceBuffer spheres; // float4 bounding sphere per record (rayhierarchy)
    pbg::DeviceBuffer clusters; // float4 sphere per kClusterTris consecutive records (rayhierarchy)
    pbg::DeviceBuffer tri_pos; // original index -> record position
    int64_t bvh_nodes = 0;
    int bvh_depth = 0;
    int32_t unculled = 0;      // records [0, unculled) are tested by every ray
    int rh_groups = 1;         // triangle groups per rayhierarchy traversal (grows on overflow)
    int walk_hint = -1;        // ray-bvh: 1 = incoherent batch, 0 = coherent, -1 = infer
    pbg::Tunables tune;        // launch shapes (pbg_autotune)
    bool host_call = false;    // inside pbg_intersect / pbg_occluded (host buffers)
    std::vector<pbg::BvhNode> host_nodes;  // ray-bvh tree, kept for the learned clusters
    std::vector<int32_t> host_order;
    struct pbg::Learner* learn = nullptr;
    struct pbg::RenderBuffers* render_bufs = nullptr;  // pbg_render's frame buffers, kept across frames
    int64_t image_w = 0, image_h = 0;  // ray-image layout from pbg_preprocess (0 = none)
    float scene_lo[3] = {0, 0, 0}, scene_hi[3] = {0, 0, 0};
    pbg::DeviceBuffer err;     // int[4] device status words
    int* mbox_host = nullptr;  // mapped pinned words the host reads status through
    int* mbox_dev = nullptr;   // the same words as the device addresses them
    uint32_t mbox_seq = 0;     // sequence number of the last publication
    pbg::DeviceBuffer workc;   // uint64[8] traversal work counters (profiling level 2)
    pbg::Work work;
    pbg::Work alt;             // the second part's buffers in two-part host shadow calls
    pbg_counters counters{};
    pbg::Profiler prof;
};

namespace pbg {

// Kernel launchers (one translation unit each).
int launch_pack_rays(pbg_scene* s, const float* stage, int64_t n, float4* o, float4* d,
                     cudaStream_t st);
int naive_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                  int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st);
int naive_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                   uint8_t* occ, cudaStream_t st);
int bvh_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st);
int bvh_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                 uint8_t* occ, cudaStream_t st);
int bvh_nearest_hinted(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                       const uint16_t* hint, int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st);
int bvh_occluded_hinted(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                        const uint16_t* hint, uint8_t* occ, int32_t* occluders, cudaStream_t st);
// Walks 5 and 6 (coop) over the eight-wide tree; ensure_wide builds it on
// first use and sets *available = false when the scene keeps the two-wide
// walks.
int ensure_wide(pbg_scene* s, bool* available, cudaStream_t st);
// The collapse on the device from a device-built tree (its levels in
// s->bvh_levels): fills s->wide and src (per record position of the wide
// copy, the record's position in the two-wide order); *fits = false when the
// tree does not fit the wide format.
int collapse_wide_device(pbg_scene* s, bool* fits, DeviceBuffer& src, int64_t* nwide, cudaStream_t st);
int wide_nearest(pbg_scene* s, bool coop, const float4* o, const float4* d, const uint8_t* valid,
                 const int32_t* perm, int64_t n, int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st);
int wide_occluded(pbg_scene* s, bool coop, const float4* o, const float4* d, const uint8_t* valid,
                  const int32_t* perm, int64_t n, int32_t* occluders, uint8_t* occ, cudaStream_t st);
int rh_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
               int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st);
int rh_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                uint8_t* occ, cudaStream_t st);
// The accelerator's batch query (device rays and results on st).
int run_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st);
int run_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid, int64_t n,
                 uint8_t* occ, cudaStream_t st);
int hit_geometry(pbg_scene* s, const float4* o, const float4* d, const int32_t* prim,
                 const float* t, const float* b1, const float* b2, int64_t n, float* out14,
                 cudaStream_t st);
int upload_triangles(pbg_scene* s, const float* tri9_host, const int32_t* order);
// TriRec[i] from device vertices tri9_dev[order_dev[i]] (record index = local triangle index).
int launch_build_tris(const float* tri9_dev, const int32_t* order_dev, int64_t ntri, TriRec* out,
                      cudaStream_t st);
void cluster_triangle_order(const float* tri9, int64_t ntri, std::vector<int32_t>* order);
int check_device_status(pbg_scene* s, cudaStream_t st);
void render_free(pbg_scene* s);
// Copies count (< kMailboxWords) device words to the host: a one-warp
// kernel stores them into mapped pinned memory and the host polls for them.
// No copy-engine transfer is involved, so the read never queues behind
// large transfers the caller has in flight.
constexpr int kMailboxWords = 16;
int read_device_words(pbg_scene* s, const int* dev, int count, int* out, cudaStream_t st);
// The two halves of read_device_words: work enqueued between them runs while
// the host waits for the words.
int publish_device_words(pbg_scene* s, const int* dev, int count, int* seq, cudaStream_t st);
int wait_device_words(pbg_scene* s, int seq, int count, int* out, cudaStream_t st);

// Stage timing around one launch (no-ops unless profiling is on); stages:
// 0 ray sort, 1 hierarchy build, 2 traversal, 3 finalize / other.
enum { kStageSort = 0, kStageBuild = 1, kStageTraverse = 2, kStageOther = 3 };
void prof_begin(pbg_scene* s, cudaStream_t st);
void prof_end(pbg_scene* s, cudaStream_t st, int stage, int launches);

}  // namespace pbg
