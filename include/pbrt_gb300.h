/*
 * pbrt_gb300.h -- C ABI of the GB300 ray-batch intersection library
 * (libpbrtgb300.so).
 *
 * This is the boundary the pbrt-v2 fork's batch accelerators call instead of
 * their OpenCL host code.  Each entry point names the reference interface it
 * replaces (paths relative to the fork's src/).  Plain pointers and sizes
 * only; every function returns a pbg status (0 = success) and never aborts;
 * pbg_last_error() gives the text of the last failure on the calling thread.
 *
 * Data layout
 *   triangles  float[9*ntri], v0.xyz v1.xyz v2.xyz per triangle in world
 *              space, the packing of accelerators/naive.cpp:59-101
 *              ("vertices[9*n]"); optional uv float[6*ntri] (u,v per vertex,
 *              shapes/trianglemesh.h:81-95; NULL = pbrt's defaults).
 *   host rays  pbg_rays: eight float arrays (o.xyz, d.xyz, mint, maxt; the
 *              fields of Ray, core/geometry.h:314-336) and an optional
 *              validity mask (the `hit` array of the batch calls; 0 = skip).
 *   device rays two arrays of 16-byte records: o4[i] = (ox, oy, oz, mint),
 *              d4[i] = (dx, dy, dz, maxt), 16-byte aligned.
 *   hits       prim (int32, index into the triangle array, -1 = miss), t, b1,
 *              b2; prim/t/b1/b2 equal pbrt's Triangle::Intersect
 *              (shapes/trianglemesh.cpp:119-156) looped over the triangles
 *              in index order: the least t, and on an exact tie in t the
 *              highest index.
 *   occlusion  uint8 0/1 per ray (the batch API's '0'/'1' chars are
 *              produced by the adapter).
 *
 * Threading: calls on one scene must be serialised by the caller (the
 * reference serialises its device with Semaphore(1), naive.cpp:109); distinct
 * scenes may be used from distinct threads.
 */
#ifndef PBRT_GB300_H
#define PBRT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define PBG_OK 0
#define PBG_ERR_INVALID_ARGUMENT 1
#define PBG_ERR_CUDA 2
#define PBG_ERR_OUT_OF_MEMORY 3
#define PBG_ERR_DEVICE_TIMEOUT 4 /* a bounded device-side wait gave up */
#define PBG_ERR_NO_DEVICE 5
#define PBG_ERR_UNSUPPORTED 6
#define PBG_ERR_INTERNAL 7

/* Accelerator kinds: the scene-file names of api.cpp:586-591. */
#define PBG_ACCEL_NAIVE 0        /* Accelerator "naive"        */
#define PBG_ACCEL_RAYHIERARCHY 1 /* Accelerator "rayhierarchy" */
#define PBG_ACCEL_RAYBVH 2       /* Accelerator "ray-bvh"      */

typedef struct pbg_scene pbg_scene;

/* Construction parameters.  Names follow the scene-file parameters of
 * rayhierarchy.cpp:1331-1339 and rayBVH.cpp:1328-1335; 0 selects the
 * library's tuned default. */
typedef struct pbg_params {
    int32_t chunk_x;      /* "chunkXSize": rays per leaf along x (rayhierarchy) */
    int32_t chunk_y;      /* "chunkYSize" */
    int32_t height;       /* "height": ray-hierarchy levels */
    int32_t bvh_height;   /* "BVHheight": levels of the BVH cut for ray-bvh */
    int32_t max_bvh_prim; /* "maxBVHPrim": triangles per BVH leaf */
    int32_t device;       /* CUDA device ordinal */
    int32_t ray_sort;     /* ray-bvh: 1 = walk each batch in 6-D Morton order
                           * (helps incoherent bounce rays), 0 = caller order */
    int32_t rh_cluster_levels; /* rayhierarchy: hierarchy levels walked by clusters of
                                * 32 triangles before they split (0 = down to the
                                * leaves' parents, < 0 = no clusters) */
    int32_t walk;         /* ray-bvh traversal: 0 = automatic (what pbg_autotune
                           * chose for the batch class, else 6 for bounce
                           * batches -- nearest hit with a validity mask, and
                           * the renderer's bounces >= 1 --, 4 for other
                           * nearest-hit batches, 5 for other any-hit ones),
                           * 1 = one thread per ray, 2 = persistent warps refilled
                           * from a ray counter, 3 = co-traversal of the ray
                           * hierarchy's 32-ray leaves with the BVH, one warp
                           * packet per leaf (rayBVH.cpp:615-836), 4 = the same
                           * packets over the batch in the caller's order,
                           * 5 = persistent warps over the tree collapsed to
                           * eight children per node (built on the first
                           * such batch; a tree outside that format keeps
                           * walk 2), 6 = the same with each warp's triangle
                           * tests spread over all its lanes.  Every walk
                           * returns the same results bit for bit. */
    int32_t bvh_build;    /* ray-bvh: 0 = build the SAH tree on the device,
                           * 1 = on the host (the same splits; numbered depth
                           * first instead of breadth first) */
    int32_t rh_queue_pairs; /* rayhierarchy: capacity of each ray/node pair queue
                             * in pairs (0 = 2^25; at least 4096).  Three such
                             * buffers of 8, 8 and 4 bytes a pair are held; a
                             * batch whose pairs overflow them is traced again
                             * with the triangles split into more groups. */
    int32_t reserved[5];
} pbg_params;

typedef struct pbg_rays {
    const float *ox, *oy, *oz;
    const float *dx, *dy, *dz;
    const float *mint, *maxt;
    const uint8_t* valid; /* may be NULL: every ray valid */
} pbg_rays;

typedef struct pbg_hits {
    int32_t* prim;
    float* t;
    float* b1;
    float* b2;
} pbg_hits;

typedef struct pbg_counters {
    uint64_t rays_nearest;    /* rays traced by intersect calls */
    uint64_t rays_occluded;   /* rays traced by occluded calls */
    uint64_t calls;
    uint64_t bvh_nodes;       /* nodes of the scene's BVH (ray-bvh) */
    uint64_t kernel_launches; /* kernels this scene has launched */
    uint64_t timed_launches[4]; /* launches timed per stage (profiling on) */
    /* Work counted by the traversal kernels at profiling level 2: [0] node
     * (or box) tests, [1] leaves visited, [2] ray/triangle filter tests,
     * [3] exact tests, [4] exact tests that hit, [5] filter tests that went
     * past the first barycentric check (ray-bvh walks).  Zero otherwise. */
    uint64_t work[6];
    /* rayhierarchy shadow batches traced in the kept origin order of the
     * previous batch, and batches traced again because their origins or
     * validity differed from it (the kept order is taken before the
     * comparison's answer is read). */
    uint64_t origin_reuses;
    uint64_t origin_reruns;
    /* rayhierarchy batches traced again with more triangle groups because a
     * pair queue overflowed (the scene keeps the larger grouping) */
    uint64_t queue_reruns;
    /* Device time per stage in ms while profiling is on (CUDA events around
     * each launch on its stream): [0] ray sort, [1] hierarchy build,
     * [2] traversal (the intersection kernels), [3] finalize / other. */
    double stage_ms[4];
    /* ray-bvh walks 5 and 6: nodes of the eight-wide tree (0 until the first
     * such batch builds it) and the host wall time of that build, ms
     * (collapse of the two-wide tree on the host cores, uploads) */
    uint64_t wide_nodes;
    double wide_build_ms;
} pbg_counters;

/* Library version, e.g. "pbrt-gb300 1.0 (sm_103a)". */
const char* pbg_version(void);
const char* pbg_status_string(int status);
/* Text of the last failure on the calling thread ("" if none). */
const char* pbg_last_error(void);
/* Number of CUDA devices visible (0 when none); never fails. */
int pbg_device_count(void);

/* Builds the device-resident scene for one accelerator.  Replaces the
 * constructors NaiveAccel::NaiveAccel (accelerators/naive.cpp:18-110),
 * RayHieararchy::RayHieararchy (accelerators/rayhierarchy.cpp:35-227) and
 * RayBVH::RayBVH (accelerators/rayBVH.cpp:31-165), and the BVH they upload
 * (rayBVH.cpp:204-276).  params may be NULL.  ntri may be 0. */
int pbg_scene_create(const float* tri9, const float* uv6, int64_t ntri, int32_t accel,
                     const pbg_params* params, pbg_scene** out);
/* Replaces the accelerators' destructors (naive.cpp:112-121). */
void pbg_scene_destroy(pbg_scene* scene);

/* The scene from pbrt's mesh arrays instead of packed triangles: P
 * [nverts][3] positions (world space), indices [ntri][3] (TriangleMesh
 * vertexIndex), uv [nverts][2] or NULL (TriangleMesh uvs).  Host arrays; the
 * triangles are gathered on the device (the packing of
 * accelerators/naive.cpp:59-101 without the host loop), and naive and
 * ray-bvh scenes are then built there too; a rayhierarchy scene orders its
 * records on the host, so it is gathered there.  Same triangle indices and
 * results as pbg_scene_create on the packed triangles.  An index outside
 * [0, nverts) is PBG_ERR_INVALID_ARGUMENT.  No counterpart in the reference. */
int pbg_scene_create_mesh(const float* P, int64_t nverts, const int32_t* indices, int64_t ntri,
                          const float* uv, int32_t accel, const pbg_params* params, pbg_scene** out);

/* Batch size cap.  Replaces NaiveAccel::MaxRaysPerCall (naive.cpp:127-142),
 * RayHieararchy::MaxRaysPerCall (rayhierarchy.cpp:267-310) and
 * RayBVH::MaxRaysPerCall (rayBVH.cpp:279-324), which return 409600. */
int pbg_max_rays_per_call(const pbg_scene* scene, int64_t* out);

/* Declares that following batches of exactly width*height rays form a ray
 * image (ray i at x = i mod width, y = i div width), as the breadth-first
 * renderer lays them out: width = tile xRes * spp, height = tile yRes.
 * Replaces RayHieararchy::Preprocess / RayBVH::Preprocess
 * (rayhierarchy.cpp:250-265, core/primitive.h:296-297).  The ray hierarchy
 * then groups rays by 2-D image tiles; 0, 0 clears the layout. */
int pbg_preprocess(pbg_scene* scene, int64_t width, int64_t height);

/* Nearest hit of n rays, host buffers in and out (copies included).
 * Replaces the batch Intersect of naive.cpp:204-338,
 * rayhierarchy.cpp:602-813 / :816-1140 and rayBVH.cpp:615-836 / :839-1138
 * (the traversal part; the Intersection records are filled by the caller
 * from prim/t/b1/b2 and pbg_hit_geometry).  Rays with valid[i] == 0 get
 * prim = -1. */
int pbg_intersect(pbg_scene* scene, const pbg_rays* rays, int64_t n, pbg_hits* out);

/* Shadow any-hit of n rays, host buffers.  Replaces the batch IntersectP of
 * naive.cpp:357-437, rayhierarchy.cpp:1170-1326 and rayBVH.cpp:1170-1323.
 * occ[i] = 1 when a triangle is hit with t in [mint, maxt]; 0 for a ray with
 * valid[i] == 0. */
int pbg_occluded(pbg_scene* scene, const pbg_rays* rays, int64_t n, uint8_t* occ);

/* Device-resident forms: every pointer is device memory, work is enqueued
 * on `stream` (a cudaStream_t; NULL = the scene's own stream) and the call
 * returns without synchronising.  valid may be NULL. */
int pbg_intersect_device(pbg_scene* scene, const float* o4, const float* d4,
                         const uint8_t* valid, int64_t n, int32_t* prim, float* t, float* b1,
                         float* b2, void* stream);
int pbg_occluded_device(pbg_scene* scene, const float* o4, const float* d4,
                        const uint8_t* valid, int64_t n, uint8_t* occ, void* stream);

/* Nearest hit without any device allocation, for callers that cannot call
 * cudaMalloc (code running inside another framework's memory pool or
 * allocator hooks, or a host that has already committed the device's memory
 * to its own arenas).  No counterpart in the reference: its accelerators
 * always allocate OpenCL buffers per call.  Everything is device memory the
 * caller owns: tri9 (9 floats per triangle, as pbg_scene_create takes
 * them), o4/d4 rays, prim/t/b1/b2 outputs; no scene object is needed.
 * Results equal pbg_intersect_device on a naive scene.  Scratch is one
 * fixed 8 MB __device__ array inside the library, so at most 1048576 rays
 * per call (more is rejected with PBG_ERR_INVALID_ARGUMENT); every call
 * shares that array, so calls that overlap on the GPU race and must be
 * serialised.  Each call looks the array up in the calling thread's current
 * context; the first call in a context loads the library's device code and
 * should come before any stream capture.  o4 and d4 must be 16-byte aligned
 * and the other arrays 4-byte aligned (misaligned views are rejected with
 * PBG_ERR_INVALID_ARGUMENT).  stream = NULL is the legacy default stream. */
int pbg_intersect_naive_noalloc(const float* tri9, int64_t ntri, const float* o4,
                                const float* d4, int64_t n, int32_t* prim, float* t, float* b1,
                                float* b2, void* stream);

/* Differential geometry of each hit, the part of Triangle::Intersect that
 * builds the DifferentialGeometry (shapes/trianglemesh.cpp:158-190,
 * core/diffgeom.cpp:32-47) and the fork's computeDpTuTv kernel
 * (bin/cl/computeDpTuTv.cl:8-91).  out14 is [n][14] float: p.xyz,
 * dpdu.xyz, dpdv.xyz, nn.xyz, u, v; rows of misses are zero.  Host buffers. */
int pbg_hit_geometry(pbg_scene* scene, const pbg_rays* rays, const pbg_hits* hits, int64_t n,
                     float* out14);
int pbg_hit_geometry_device(pbg_scene* scene, const float* o4, const float* d4,
                            const int32_t* prim, const float* t, const float* b1,
                            const float* b2, int64_t n, float* out14, void* stream);

/* ---------------------------------------------------------------------
 * Breadth-first renderer on the device (renderers/breadth-first.cpp:18-228
 * with the batch Li of integrators/directlighting.cpp:112-145 and
 * integrators/path.cpp:43-157): camera rays of the whole image in one
 * batch, Lambertian shading, light sampling, shadow and bounce batches
 * through the scene's accelerator, film accumulation -- all on the GPU.
 * ------------------------------------------------------------------- */

/* Camera as pbrt's ProjectiveCamera holds it: RasterToCamera and the
 * (non-animated) CameraToWorld, row-major m[i][j] (core/camera.cpp:68-88,
 * cameras/perspective.cpp GenerateRayDifferential). */
typedef struct pbg_camera {
    float raster_to_camera[16];
    float camera_to_world[16];
    int32_t xres, yres;
} pbg_camera;

#define PBG_LIGHT_POINT 0 /* lights/point.cpp PointLight                         */
#define PBG_LIGHT_QUAD 1  /* an emitter on a parallelogram, sampled by area      */
#define PBG_LIGHT_MESH 2  /* lights/diffuse.cpp DiffuseAreaLight on scene triangles */
typedef struct pbg_light {
    int32_t type;
    int32_t nsamples;  /* "nsamples" of the area light (directlighting) */
    float pos[3];      /* point light position */
    float intensity[3];/* point light I, RGB */
    float quad[12];    /* parallelogram corners p0, p1, p2, p3 (p2 = p1 + p3 - p0) */
    float radiance[3]; /* area light L, RGB; a parallelogram emits on the side of
                          (p1-p0)x(p3-p0), a triangle on the side of its
                          DifferentialGeometry normal */
    int32_t first_tri; /* PBG_LIGHT_MESH: the emitter is the scene's triangles */
    int32_t ntri;      /* [first_tri, first_tri + ntri), 1..64 (its ShapeSet)  */
} pbg_light;

#define PBG_INTEGRATOR_DIRECT 0 /* SurfaceIntegrator "directlighting" */
#define PBG_INTEGRATOR_PATH 1   /* SurfaceIntegrator "path"           */
typedef struct pbg_render_params {
    int32_t integrator;
    int32_t spp_x, spp_y;   /* stratified sampler grid per pixel */
    int32_t jitter;         /* 0: sample centres (pbrt "jitter" false) */
    int32_t max_depth;      /* "maxdepth" (path: default 5) */
    int32_t reserved0;
    uint64_t seed;          /* counter-based sample stream seed */
    float albedo[3];        /* MatteMaterial Kd of every triangle */
    int32_t reserved[8];
} pbg_render_params;

typedef struct pbg_render_stats {
    uint64_t camera_rays, nearest_rays, shadow_rays, bounces;
    double ms_total;
} pbg_render_stats;

/* Renders the image; rgb receives [yres][xres][3] floats (host memory),
 * ImageFilm's XYZ accumulation and box filter (film/image.cpp).  stats may
 * be NULL.  Sample values come from a counter-based hash of
 * (params->seed, sample, dimension). */
int pbg_render(pbg_scene* scene, const pbg_camera* camera, const pbg_light* lights,
               int32_t nlights, const pbg_render_params* params, float* rgb,
               pbg_render_stats* stats);

/* One breadth-first task's sample values as the reference draws them
 * (renderers/breadth-first.cpp:18-48): the samples its StratifiedSampler
 * produced and the continuation of the task's RNG.  Host arrays.
 *   image_xy  [count][2]  Sample::imageX, imageY, in the task's order
 *   dims      [count][ndims], per sample:
 *             directlighting: 6 values per light sample, lights in order and
 *               each light's nsamples in order: LightSample uPos[0], uPos[1],
 *               uComponent, BSDFSample uDir[0], uDir[1], uComponent (the
 *               integrator's arrays, integrators/directlighting.cpp:45-62)
 *             path: 10 values for each of the bounces 0-2: light choice,
 *               LightSample uPos[0..1], uComponent, BSDFSample uDir[0..1],
 *               uComponent, the path's BSDFSample uDir[0..1], uComponent
 *               (integrators/path.cpp:31-38)
 *   rng       [nrng] the task RNG's RandomFloat draws after the sampler's;
 *             path bounces from 3 on consume them as the batch integrator
 *             does: 7 per ray of the task for UniformSampleOneLight, then 3
 *             per ray that hit (4 after bounce 3, Russian roulette)
 * count camera rays are traced; a sample adds to the pixels of ImageFilm's
 * box-filter footprint around (imageX, imageY).  A path vertex whose sampled
 * direction the BSDF rejects ends the render with PBG_ERR_UNSUPPORTED (the
 * reference would trace that ray again unchanged). */
typedef struct pbg_sample_stream {
    int64_t count;
    const float* image_xy;
    const float* dims;
    int32_t ndims;
    int32_t reserved;
    const float* rng;
    int64_t nrng;
} pbg_sample_stream;

/* pbg_render with the reference's sample stream instead of the hash (no
 * counterpart in the reference: its renderer draws these values itself). */
int pbg_render_stream(pbg_scene* scene, const pbg_camera* camera, const pbg_light* lights,
                      int32_t nlights, const pbg_render_params* params,
                      const pbg_sample_stream* stream, float* rgb, pbg_render_stats* stats);

/* ---------------------------------------------------------------------
 * Many scenes in one launch.  No counterpart in the reference (one scene,
 * one batch per call).  A scene set holds up to 4096 ray-bvh scenes; one
 * trace call answers nearest-hit and any-hit queries of every scene with
 * one persistent kernel pulling warp-sized work items from a global queue.
 * The launch sequence is captured once as a CUDA graph and replayed while
 * the same arrays and parameters are passed; the tile, grid and block
 * shape come from the built-in autotuner unless given.
 * ------------------------------------------------------------------- */
typedef struct pbg_sceneset pbg_sceneset;

typedef struct pbg_batch_params {
    int32_t tile;        /* rays per work item, multiple of 32 (0 = tuned) */
    int32_t ctas_per_sm; /* persistent CTAs per SM (0 = tuned) */
    int32_t threads;     /* threads per CTA, multiple of 32 (0 = tuned) */
    int32_t use_graph;   /* 1 = capture and replay a CUDA graph (default 1) */
    int32_t walk;        /* 1 = warps take work items of `tile` rays, 2 = each lane
                          * refills from one counter over all rays, 3 = the same
                          * over every scene's eight-wide tree (one launch per
                          * query kind, 128 threads), 4 = 3 with each warp's
                          * triangle tests spread over its lanes (0 = tuned) */
    int32_t reserved[7];
} pbg_batch_params;

typedef struct pbg_batch_stats {
    double ms;                       /* device time of the call's launch sequence */
    double scene_ms_p50, scene_ms_p99; /* per-scene completion times since launch */
    uint64_t rays;
    int32_t tile, ctas_per_sm, threads, graph_replayed;
    int32_t walk, reserved;
} pbg_batch_stats;

int pbg_sceneset_create(int32_t nscenes, const float* const* tri9, const int64_t* ntri,
                        int32_t device, pbg_sceneset** out);
void pbg_sceneset_destroy(pbg_sceneset* set);
/* Scene k's nearest-hit rays are o4n/d4n[near_offsets[k] .. near_offsets[k+1])
 * (device records as for pbg_intersect_device, offsets host int64 with
 * nscenes + 1 entries) with results prim/t/b1/b2 at the same indices
 * (triangle indices local to scene k); likewise any-hit rays o4s/d4s with
 * occ.  Either query set may be empty (NULL arrays, zero offsets).
 * scene_ms (host, nscenes entries, may be NULL) receives each scene's
 * completion time.  params may be NULL (tuned).  Synchronises when stats or
 * scene_ms are requested. */
int pbg_sceneset_trace(pbg_sceneset* set, const float* o4n, const float* d4n,
                       const int64_t* near_offsets, int32_t* prim, float* t, float* b1, float* b2,
                       const float* o4s, const float* d4s, const int64_t* occ_offsets, uint8_t* occ,
                       const pbg_batch_params* params, pbg_batch_stats* stats, double* scene_ms,
                       void* stream);
/* Times the candidate shapes on these queries and keeps the fastest as the
 * set's tuned parameters (written to *best if not NULL). */
int pbg_sceneset_autotune(pbg_sceneset* set, const float* o4n, const float* d4n,
                          const int64_t* near_offsets, int32_t* prim, float* t, float* b1,
                          float* b2, const float* o4s, const float* d4s, const int64_t* occ_offsets,
                          uint8_t* occ, pbg_batch_params* best, void* stream);

/* ---------------------------------------------------------------------
 * Learned traversal ordering (Accelerator "ray-bvh" only).  No counterpart
 * in the reference.  An MLP (105 ray features -> 64 -> 64 -> 256 logits,
 * BF16 weights, FP32 accumulation, tcgen05 kernels) predicts which of the
 * 256 top clusters of the BVH holds a ray's first hit; the traversal visits
 * that cluster first and then runs the full exact walk, so hits and
 * occlusion are identical with the ordering on or off.  Training is online,
 * on the records the accelerator collects from its own batches: first-hit
 * clusters of nearest-hit rays, and the clusters of the occluders any-hit
 * walks find (a shadow ray whose guess holds an occluder stops there).
 * ------------------------------------------------------------------- */
typedef struct pbg_learn_params {
    int32_t batch;            /* records per SGD step (multiple of 128; 0 = 8192) */
    int32_t steps_per_train;  /* SGD steps per pbg_learn_train call (0 = 8) */
    float lr;                 /* learning rate (0 = 0.05) */
    float momentum;           /* (0 = 0.9) */
    int32_t records;          /* training records kept, ring buffer (0 = 262144) */
    float margin;             /* a ray walks its predicted cluster first only when the
                               * top logit leads the second by at least this (0 = 1.0;
                               * < 0 = always) */
    uint64_t seed;            /* weight initialisation */
    int32_t queries;          /* batches the ordering serves and learns from:
                               * 1 nearest-hit (first-hit clusters), 2 any-hit
                               * (occluder clusters), 3 both (0 = 3) */
    int32_t reserved[7];
} pbg_learn_params;

typedef struct pbg_learn_stats {
    uint64_t trained_steps, records;
    float last_loss, last_accuracy; /* of the last SGD step (top-1 cluster) */
    double infer_ms, train_ms;      /* device time spent so far */
} pbg_learn_stats;

/* on = 1 builds the clusters and the network (params may be NULL); a later
 * call with on = 1 switches the ordering back on and updates the given
 * (non-zero) batch, steps, learning rate, momentum, margin and queries,
 * keeping the trained weights and the records.  on = 0 switches the
 * ordering off (the plain kernels run). */
int pbg_learn_enable(pbg_scene* scene, int32_t on, const pbg_learn_params* params);
/* Runs SGD steps on the collected records (steps <= 0: steps_per_train). */
int pbg_learn_train(pbg_scene* scene, int32_t steps);
int pbg_learn_get_stats(pbg_scene* scene, pbg_learn_stats* out);
/* Parameters as FP32 host arrays in the order W1 [64 x 112], b1 [64],
 * W2 [64 x 64], b2 [64], W3 [256 x 64], b3 [256] (27,648 + 384 floats):
 * read (get = 1) or write (get = 0). */
int pbg_learn_params_io(pbg_scene* scene, float* params, int32_t get);
/* One forward + backward pass on host records x [B x 112] (float, rounded
 * to BF16 as the network sees them) and labels [B] (B % 128 == 0): writes
 * the FP32 gradients in the layout of pbg_learn_params_io, and the loss.
 * Leaves the parameters unchanged; for checking the tensor-core backward
 * pass against a CPU reference. */
int pbg_learn_gradients(pbg_scene* scene, const float* x, const int32_t* labels, int32_t B,
                        float* grads, float* loss);

/* Cluster hints (Accelerator "ray-bvh").  No counterpart in the reference.
 * The learned ordering's clusters are the 256 subtrees of the BVH's top cut;
 * a caller that knows a likely cluster per ray (the previous frame's hit of
 * the same pixel, the occluder of a neighbouring shadow ray, its own model)
 * passes it and the walk visits that subtree first.  Results are identical
 * with or without hints.  All arrays are device memory on `stream`.
 *   pbg_clusters_of_device     cluster[i] of triangle prim[i] (0..255, or
 *                              0xffff for -1 and triangles outside the cut)
 *   pbg_intersect_hinted_device / pbg_occluded_hinted_device
 *                              hint[i] = the cluster to walk first, 0xffff =
 *                              none (hint NULL: the learned ordering, if on);
 *                              occluders (may be NULL) receives the triangle
 *                              that blocked each any-hit ray, or -1 */
int pbg_clusters_of_device(pbg_scene* scene, const int32_t* prim, int64_t n, uint16_t* cluster,
                           void* stream);
int pbg_intersect_hinted_device(pbg_scene* scene, const float* o4, const float* d4,
                                const uint8_t* valid, int64_t n, const uint16_t* hint, int32_t* prim,
                                float* t, float* b1, float* b2, void* stream);
int pbg_occluded_hinted_device(pbg_scene* scene, const float* o4, const float* d4,
                               const uint8_t* valid, int64_t n, const uint16_t* hint, uint8_t* occ,
                               int32_t* occluders, void* stream);

/* Tensor-core GEMM used by the learned traversal ordering, exposed for
 * checking: C[M x N] (+)= A[M x K] * B[N x K]^T with A, B row-major BF16
 * (raw 16-bit patterns) and C row-major FP32, all device memory; tcgen05
 * MMAs with FP32 accumulation in tensor memory.  M % 128 == 0,
 * 16 <= N <= 256 with N % 16 == 0, K % 16 == 0.  Synchronises the stream.
 * No counterpart in the reference (it has no learned component). */
int pbg_tc_gemm_bf16(const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t N,
                     int32_t K, int32_t accumulate, void* stream);

/* Launch-shape autotuner (replaces picking chunkXSize / chunkYSize /
 * height by hand, rayhierarchy.cpp:1329-1348).  Traces the device batch
 * o4/d4 (16-byte ray records, valid may be NULL) with every candidate shape
 * of the scene's accelerator -- naive: CTAs per SM of the triangle splits
 * (2, 4, 8, 16); rayhierarchy: nodes of the seed level (64, 256, 1024) x
 * CTAs per SM of the grid-stride kernels (16, 32), per query kind; ray-bvh:
 * walk 1-6 (pbg_params.walk) for this batch class -- times each on `stream`
 * (best of `reps` after a warm-up run), checks that every candidate's
 * results equal the first one's bit for bit (else PBG_ERR_INTERNAL and the
 * scene keeps its shapes), and keeps the fastest for later calls.
 * query: bit 0 = any-hit (else nearest hit), bit 1 = an incoherent batch
 * (bounce rays; ray-bvh keeps a walk per any-hit/incoherent class).
 * Allocates scratch for two result sets while it runs; synchronises. */
typedef struct pbg_tune_result {
    int32_t ncandidates;
    int32_t best;            /* index of the candidate kept */
    int32_t setting[16][3];  /* naive {ctas}, rayhierarchy {seed nodes, grid}, ray-bvh {walk 1-6} */
    float ms[16];            /* device time of the batch with each candidate */
    uint64_t mismatches;     /* results that differed from the first candidate's (0) */
} pbg_tune_result;
int pbg_autotune(pbg_scene* scene, const float* o4, const float* d4, const uint8_t* valid, int64_t n,
                 int32_t query, int32_t reps, pbg_tune_result* out, void* stream);

/* Counters and per-stage device times (replaces the GPU_TIMES / STAT_*
 * printouts, core/GPUparallel.h:532-538 and rayhierarchy.cpp:229-239).
 * Reading them synchronises the scene's pending timing events. */
int pbg_stats(pbg_scene* scene, pbg_counters* out);
/* Turns per-stage event timing on (1) or off (0) and clears the stage
 * times and work counters.  Off by default: timing adds two event records
 * per launch.  Level 2 also counts traversal work (counters.work) with a
 * counting variant of the traversal kernels. */
int pbg_profile(pbg_scene* scene, int on);

#ifdef __cplusplus
}
#endif

#endif /* PBRT_GB300_H */
