// pbg_api.cu -- the C ABI (include/pbrt_gb300.h): scene lifetime, batch
// calls with host or device buffers, hit geometry and counters.
//
// Host-side duties of the reference accelerators that live here:
//   - packing triangles once at construction (accelerators/naive.cpp:59-101,
//     rayhierarchy.cpp:158-205) -> TriRec records built on the device;
//   - AoS -> SoA ray packing per batch (naive.cpp:224-262,
//     rayhierarchy.cpp:833-853) -> one H2D copy of the caller's SoA rows and
//     a pack kernel into 16-byte records;
//   - reading back tHit/index and computeDpTuTv results
//     (rayhierarchy.cpp:1048-1091) -> D2H copies of prim/t/b1/b2 and of the
//     hit geometry.
// Errors become status codes; nothing aborts (the reference calls Severe(),
// core/error.cpp:130).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "pbg_internal.h"
#include "pbg_learn.h"
#include "pbg_tma.cuh"

namespace pbg {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

int cuda_status(cudaError_t e, const char* what) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    set_last_error(buf);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // clear the sticky-free allocation error
        return PBG_ERR_OUT_OF_MEMORY;
    }
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PBG_ERR_NO_DEVICE;
    return PBG_ERR_CUDA;
}

int ensure(DeviceBuffer& b, size_t bytes) {
    if (bytes <= b.bytes && b.ptr) return PBG_OK;
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&b.ptr, want);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        return cuda_status(e, "cudaMalloc");
    }
    b.bytes = want;
    return PBG_OK;
}

void release(DeviceBuffer& b) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

// ---------------------------------------------------------------- kernels

// TriRec from original vertices; e1, e2 rounded as pbrt rounds p2 - p1 and
// p3 - p1 (shapes/trianglemesh.cpp:127-128).  order (may be NULL) lists the
// original index of each record; pos receives the inverse map.
__global__ void build_tris_kernel(const float* __restrict__ tri9, const int32_t* __restrict__ order,
                                  int64_t ntri, TriRec* __restrict__ out, int32_t* __restrict__ pos) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntri) return;
    const int32_t src = order ? order[i] : (int32_t)i;
    const float* v = tri9 + 9 * (int64_t)src;
    const float p1x = v[0], p1y = v[1], p1z = v[2];
    const float e1x = __fsub_rn(v[3], p1x), e1y = __fsub_rn(v[4], p1y), e1z = __fsub_rn(v[5], p1z);
    const float e2x = __fsub_rn(v[6], p1x), e2y = __fsub_rn(v[7], p1y), e2z = __fsub_rn(v[8], p1z);
    TriRec r;
    r.a = make_float4(p1x, p1y, p1z, fabsf(e1x) + fabsf(e1y) + fabsf(e1z));
    r.b = make_float4(e1x, e1y, e1z, fabsf(e2x) + fabsf(e2y) + fabsf(e2z));
    r.c = make_float4(e2x, e2y, e2z, __int_as_float(src));
    out[i] = r;
    if (pos) pos[src] = (int32_t)i;
}

// Caller SoA rows (8 x n floats, one staging block) -> 16-byte records.
__global__ void pack_rays_kernel(const float* __restrict__ stage, int64_t n, float4* __restrict__ o,
                                 float4* __restrict__ d) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    o[i] = make_float4(stage[i], stage[n + i], stage[2 * n + i], stage[6 * n + i]);
    d[i] = make_float4(stage[3 * n + i], stage[4 * n + i], stage[5 * n + i], stage[7 * n + i]);
}

__device__ __forceinline__ void xcross3(float ax, float ay, float az, float bx, float by, float bz,
                                        float* x, float* y, float* z) {
    *x = xcross(ay, bz, az, by);
    *y = xcross(az, bx, ax, bz);
    *z = xcross(ax, by, ay, bx);
}

// DifferentialGeometry of a hit (shapes/trianglemesh.cpp:158-190,
// core/diffgeom.cpp:32-47, core/geometry.h:512-522), pbrt's rounding.
__global__ void hit_geometry_kernel(const float* __restrict__ tri9, const float* __restrict__ uv6,
                                    const float4* __restrict__ ro, const float4* __restrict__ rd,
                                    const int32_t* __restrict__ prim, const float* __restrict__ tt,
                                    const float* __restrict__ b1v, const float* __restrict__ b2v,
                                    int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* g = out + 14 * i;
    const int32_t p = prim[i];
    if (p < 0) {
        for (int k = 0; k < 14; ++k) g[k] = 0.f;
        return;
    }
    const float* v = tri9 + 9 * (int64_t)p;
    float u[3][2];
    if (uv6) {
        const float* q = uv6 + 6 * (int64_t)p;
        u[0][0] = q[0]; u[0][1] = q[1]; u[1][0] = q[2]; u[1][1] = q[3]; u[2][0] = q[4]; u[2][1] = q[5];
    } else {
        u[0][0] = 0.f; u[0][1] = 0.f; u[1][0] = 1.f; u[1][1] = 0.f; u[2][0] = 1.f; u[2][1] = 1.f;
    }
    const float du1 = __fsub_rn(u[0][0], u[2][0]), du2 = __fsub_rn(u[1][0], u[2][0]);
    const float dv1 = __fsub_rn(u[0][1], u[2][1]), dv2 = __fsub_rn(u[1][1], u[2][1]);
    float dp1[3], dp2[3], dpdu[3], dpdv[3];
    for (int k = 0; k < 3; ++k) {
        dp1[k] = __fsub_rn(v[k], v[6 + k]);
        dp2[k] = __fsub_rn(v[3 + k], v[6 + k]);
    }
    const float det = __fsub_rn(__fmul_rn(du1, dv2), __fmul_rn(dv1, du2));
    if (det == 0.f) {
        float e1[3], e2[3];
        for (int k = 0; k < 3; ++k) {
            e1[k] = __fsub_rn(v[3 + k], v[k]);
            e2[k] = __fsub_rn(v[6 + k], v[k]);
        }
        float nx, ny, nz;
        xcross3(e2[0], e2[1], e2[2], e1[0], e1[1], e1[2], &nx, &ny, &nz);
        const float inv = __frcp_rn(__fsqrt_rn(xdot(nx, ny, nz, nx, ny, nz)));
        const float v1x = __fmul_rn(nx, inv), v1y = __fmul_rn(ny, inv), v1z = __fmul_rn(nz, inv);
        if (fabsf(v1x) > fabsf(v1y)) {
            const float il = __frcp_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(v1x, v1x), __fmul_rn(v1z, v1z))));
            dpdu[0] = __fmul_rn(-v1z, il); dpdu[1] = 0.f; dpdu[2] = __fmul_rn(v1x, il);
        } else {
            const float il = __frcp_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(v1y, v1y), __fmul_rn(v1z, v1z))));
            dpdu[0] = 0.f; dpdu[1] = __fmul_rn(v1z, il); dpdu[2] = __fmul_rn(-v1y, il);
        }
        xcross3(v1x, v1y, v1z, dpdu[0], dpdu[1], dpdu[2], &dpdv[0], &dpdv[1], &dpdv[2]);
    } else {
        const float invdet = __frcp_rn(det);
        for (int k = 0; k < 3; ++k) {
            dpdu[k] = __fmul_rn(__fsub_rn(__fmul_rn(dv2, dp1[k]), __fmul_rn(dv1, dp2[k])), invdet);
            dpdv[k] = __fmul_rn(__fadd_rn(__fmul_rn(-du2, dp1[k]), __fmul_rn(du1, dp2[k])), invdet);
        }
    }
    const float b1 = b1v[i], b2 = b2v[i], t = tt[i];
    const float b0 = __fsub_rn(__fsub_rn(1.f, b1), b2);
    const float tu = __fadd_rn(__fadd_rn(__fmul_rn(b0, u[0][0]), __fmul_rn(b1, u[1][0])), __fmul_rn(b2, u[2][0]));
    const float tv = __fadd_rn(__fadd_rn(__fmul_rn(b0, u[0][1]), __fmul_rn(b1, u[1][1])), __fmul_rn(b2, u[2][1]));
    const float4 o = ro[i], d = rd[i];
    g[0] = __fadd_rn(o.x, __fmul_rn(d.x, t));
    g[1] = __fadd_rn(o.y, __fmul_rn(d.y, t));
    g[2] = __fadd_rn(o.z, __fmul_rn(d.z, t));
    float nx, ny, nz;
    xcross3(dpdu[0], dpdu[1], dpdu[2], dpdv[0], dpdv[1], dpdv[2], &nx, &ny, &nz);
    const float inv = __frcp_rn(__fsqrt_rn(xdot(nx, ny, nz, nx, ny, nz)));
    g[3] = dpdu[0]; g[4] = dpdu[1]; g[5] = dpdu[2];
    g[6] = dpdv[0]; g[7] = dpdv[1]; g[8] = dpdv[2];
    g[9] = __fmul_rn(nx, inv); g[10] = __fmul_rn(ny, inv); g[11] = __fmul_rn(nz, inv);
    g[12] = tu;
    g[13] = tv;
}

int launch_pack_rays(pbg_scene* s, const float* stage, int64_t n, float4* o, float4* d,
                     cudaStream_t st) {
    (void)s;
    if (n <= 0) return PBG_OK;
    prof_begin(s, st);
    pack_rays_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(stage, n, o, d);
    prof_end(s, st, kStageOther, 1);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

int hit_geometry(pbg_scene* s, const float4* o, const float4* d, const int32_t* prim,
                 const float* t, const float* b1, const float* b2, int64_t n, float* out14,
                 cudaStream_t st) {
    if (n <= 0) return PBG_OK;
    prof_begin(s, st);
    hit_geometry_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(
        (const float*)s->tri9.ptr, (const float*)s->uv6.ptr, o, d, prim, t, b1, b2, n, out14);
    prof_end(s, st, kStageOther, 1);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

static cudaEvent_t prof_event(pbg_scene* s) {
    cudaEvent_t e = nullptr;
    if (!s->prof.pool.empty()) {
        e = s->prof.pool.back();
        s->prof.pool.pop_back();
        return e;
    }
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

static thread_local cudaEvent_t g_open_event = nullptr;

void prof_begin(pbg_scene* s, cudaStream_t st) {
    if (!s->prof.on) return;
    g_open_event = prof_event(s);
    if (g_open_event) cudaEventRecord(g_open_event, st);
}

void prof_end(pbg_scene* s, cudaStream_t st, int stage, int launches) {
    s->counters.kernel_launches += (uint64_t)launches;
    if (!s->prof.on || !g_open_event) return;
    cudaEvent_t b = prof_event(s);
    if (!b) return;
    cudaEventRecord(b, st);
    s->prof.pending.push_back({g_open_event, b, stage});
    s->counters.timed_launches[stage] += (uint64_t)launches;
    g_open_event = nullptr;
}

static void prof_collect(pbg_scene* s) {
    for (auto& r : s->prof.pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess)
            s->counters.stage_ms[r.stage] += ms;
        else
            cudaGetLastError();
        s->prof.pool.push_back(r.a);
        s->prof.pool.push_back(r.b);
    }
    s->prof.pending.clear();
    if (s->prof.level >= 2 && s->workc.ptr) {
        unsigned long long h[8];
        if (cudaMemcpy(h, s->workc.ptr, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess)
            for (int k = 0; k < 6; ++k) s->counters.work[k] = h[k];
        else
            cudaGetLastError();
    }
}

// Stores the words, then (after a system-scope fence) the sequence number
// in the last word: a host that sees the number sees the words.
__global__ void publish_words_kernel(const int* __restrict__ src, int count, int* dst, int seq) {
    if (threadIdx.x != 0) return;
    volatile int* d = dst;
    for (int k = 0; k < count; ++k) d[k] = src[k];
    __threadfence_system();
    d[kMailboxWords - 1] = seq;
}

int publish_device_words(pbg_scene* s, const int* dev, int count, int* seq_out, cudaStream_t st) {
    if (count > kMailboxWords - 1 || !s->mbox_dev) return PBG_ERR_INVALID_ARGUMENT;
    const int seq = (int)++s->mbox_seq;  // compared as bits; wraps harmlessly
    publish_words_kernel<<<1, 32, 0, st>>>(dev, count, s->mbox_dev, seq);
    s->counters.kernel_launches++;
    PBG_CUDA(cudaGetLastError());
    *seq_out = seq;
    return PBG_OK;
}

int read_device_words(pbg_scene* s, const int* dev, int count, int* out, cudaStream_t st) {
    int seq = 0;
    const int rc = publish_device_words(s, dev, count, &seq, st);
    if (rc) return rc;
    return wait_device_words(s, seq, count, out, st);
}

int wait_device_words(pbg_scene* s, int seq, int count, int* out, cudaStream_t st) {
    // The host polls the mapped word instead of sleeping in a stream
    // synchronisation: it sees the kernel's store within microseconds, where
    // a blocking wait adds tens of microseconds of wake-up latency to every
    // call.  After 20 ms it waits on the stream instead (a long batch, or an
    // earlier failure, which the synchronisation then reports).
    const volatile int* h = s->mbox_host;
    const auto t0 = std::chrono::steady_clock::now();
    unsigned spins = 0;
    while (h[kMailboxWords - 1] != seq) {
        if ((++spins & 1023u) == 0 &&
            std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(20)) {
            PBG_CUDA(cudaStreamSynchronize(st));
            if (h[kMailboxWords - 1] != seq) {
                set_last_error("read_device_words: the status kernel did not publish");
                return PBG_ERR_INTERNAL;
            }
            break;
        }
    }
    std::atomic_thread_fence(std::memory_order_acquire);
    for (int k = 0; k < count; ++k) out[k] = h[k];
    return PBG_OK;
}

int check_device_status(pbg_scene* s, cudaStream_t st) {
    int h[4] = {0, 0, 0, 0};
    int rc = read_device_words(s, (const int*)s->err.ptr, 4, h, st);
    if (rc) return rc;
    if (h[kStatusTimeout] != 0 || h[kStatusOverflow] != 0) {
        PBG_CUDA(cudaMemsetAsync(s->err.ptr, 0, sizeof(h), st));
        char buf[160];
        snprintf(buf, sizeof(buf), "device status: %d bounded waits expired, %d stack overflows",
                 h[kStatusTimeout], h[kStatusOverflow]);
        set_last_error(buf);
        return h[kStatusTimeout] ? PBG_ERR_DEVICE_TIMEOUT : PBG_ERR_INTERNAL;
    }
    return PBG_OK;
}

// Bounding sphere of each record for the ray-hierarchy node test: box
// centre, farthest vertex, padded by 2^-20 relative and 2^-16 of the
// centre's magnitude; degenerate triangles get an infinite radius (no node
// may cull them).
static void triangle_spheres(const float* tri9, const int32_t* order, int64_t ntri,
                             std::vector<float4>* out) {
    out->resize((size_t)ntri);
    for (int64_t i = 0; i < ntri; ++i) {
        const float* v = tri9 + 9 * (int64_t)(order ? order[i] : i);
        float c[3];
        for (int a = 0; a < 3; ++a) {
            float lo = fminf(v[a], fminf(v[3 + a], v[6 + a]));
            float hi = fmaxf(v[a], fmaxf(v[3 + a], v[6 + a]));
            c[a] = 0.5f * (lo + hi);
        }
        double r = 0.0;
        for (int k = 0; k < 3; ++k) {
            double dx = (double)v[3 * k] - c[0], dy = (double)v[3 * k + 1] - c[1],
                   dz = (double)v[3 * k + 2] - c[2];
            r = fmax(r, sqrt(dx * dx + dy * dy + dz * dz));
        }
        float rr = (float)(r * (1.0 + 0x1p-20) +
                           (fabs(c[0]) + fabs(c[1]) + fabs(c[2])) * 0x1p-16 + 1e-30);
        if (triangle_degenerate(v) || !std::isfinite(rr)) rr = INFINITY;
        (*out)[(size_t)i] = make_float4(c[0], c[1], c[2], rr);
    }
}

// Bounding sphere of each run of kClusterTris consecutive records (the
// rayhierarchy's triangle clusters): the centre of the members' box, the
// radius reaching every member sphere (in double, rounded up), padded by
// 2^-10 of itself so the node test's distance slop covers every member.
static void cluster_spheres(const std::vector<float4>& sph, std::vector<float4>* out) {
    const size_t n = sph.size(), ncl = (n + kClusterTris - 1) / kClusterTris;
    out->resize(ncl);
    for (size_t k = 0; k < ncl; ++k) {
        const size_t b = k * kClusterTris, e = std::min(n, b + kClusterTris);
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        bool inf = false;
        for (size_t i = b; i < e; ++i) {
            const float4 q = sph[i];
            if (!std::isfinite(q.w) || !std::isfinite(q.x) || !std::isfinite(q.y) || !std::isfinite(q.z))
                inf = true;
            const double c[3] = {q.x, q.y, q.z};
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], c[a] - (double)q.w);
                hi[a] = std::max(hi[a], c[a] + (double)q.w);
            }
        }
        const float cx = (float)(0.5 * (lo[0] + hi[0])), cy = (float)(0.5 * (lo[1] + hi[1])),
                    cz = (float)(0.5 * (lo[2] + hi[2]));
        double r = 0.0;
        for (size_t i = b; i < e; ++i) {
            const float4 q = sph[i];
            const double dx = (double)q.x - cx, dy = (double)q.y - cy, dz = (double)q.z - cz;
            r = std::max(r, std::sqrt(dx * dx + dy * dy + dz * dz) + (double)q.w);
        }
        float rf = (float)(r * (1.0 + 0x1p-10) + 0x1p-100);
        if (inf || !std::isfinite(rf)) rf = INFINITY;
        (*out)[k] = make_float4(inf ? 0.f : cx, inf ? 0.f : cy, inf ? 0.f : cz, rf);
    }
}

int upload_triangles(pbg_scene* s, const float* tri9_host, const int32_t* order) {
    const int64_t ntri = s->ntri;
    const size_t nt = (size_t)(ntri > 0 ? ntri : 1);
    int rc;
    if ((rc = ensure(s->tri9, nt * 9 * sizeof(float))) || (rc = ensure(s->tris, nt * sizeof(TriRec))) ||
        (rc = ensure(s->tri_pos, nt * sizeof(int32_t))))
        return rc;
    if (ntri == 0) return PBG_OK;
    PBG_CUDA(cudaMemcpyAsync(s->tri9.ptr, tri9_host, (size_t)ntri * 9 * sizeof(float),
                             cudaMemcpyHostToDevice, s->stream));
    std::vector<float4> sph, csph;  // bounding spheres: the ray hierarchy's node tests only
    if (s->accel == PBG_ACCEL_RAYHIERARCHY) {
        if ((rc = ensure(s->spheres, nt * sizeof(float4)))) return rc;
        triangle_spheres(tri9_host, order, ntri, &sph);
        PBG_CUDA(cudaMemcpyAsync(s->spheres.ptr, sph.data(), (size_t)ntri * sizeof(float4),
                                 cudaMemcpyHostToDevice, s->stream));
        cluster_spheres(sph, &csph);
        if ((rc = ensure(s->clusters, csph.size() * sizeof(float4)))) return rc;
        PBG_CUDA(cudaMemcpyAsync(s->clusters.ptr, csph.data(), csph.size() * sizeof(float4),
                                 cudaMemcpyHostToDevice, s->stream));
    }
    DeviceBuffer dorder;
    if (order) {
        rc = ensure(dorder, (size_t)ntri * sizeof(int32_t));
        if (rc) return rc;
        PBG_CUDA(cudaMemcpyAsync(dorder.ptr, order, (size_t)ntri * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, s->stream));
    }
    build_tris_kernel<<<(unsigned)((ntri + 255) / 256), 256, 0, s->stream>>>(
        (const float*)s->tri9.ptr, (const int32_t*)dorder.ptr, ntri, (TriRec*)s->tris.ptr,
        (int32_t*)s->tri_pos.ptr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    release(dorder);
    if (e != cudaSuccess) return cuda_status(e, "build_tris_kernel");
    return PBG_OK;
}

int launch_build_tris(const float* tri9_dev, const int32_t* order_dev, int64_t ntri, TriRec* out,
                      cudaStream_t st) {
    if (ntri <= 0) return PBG_OK;
    build_tris_kernel<<<(unsigned)((ntri + 255) / 256), 256, 0, st>>>(tri9_dev, order_dev, ntri, out,
                                                                      nullptr);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

// ------------------------------------------------------------- dispatch

int run_nearest(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid,
                       int64_t n, int32_t* prim, float* t, float* b1, float* b2, cudaStream_t st) {
    switch (s->accel) {
        case PBG_ACCEL_NAIVE: return naive_nearest(s, o, d, valid, n, prim, t, b1, b2, st);
        case PBG_ACCEL_RAYBVH: return bvh_nearest(s, o, d, valid, n, prim, t, b1, b2, st);
        case PBG_ACCEL_RAYHIERARCHY: return rh_nearest(s, o, d, valid, n, prim, t, b1, b2, st);
    }
    set_last_error("unknown accelerator kind");
    return PBG_ERR_INVALID_ARGUMENT;
}

int run_occluded(pbg_scene* s, const float4* o, const float4* d, const uint8_t* valid,
                        int64_t n, uint8_t* occ, cudaStream_t st) {
    switch (s->accel) {
        case PBG_ACCEL_NAIVE: return naive_occluded(s, o, d, valid, n, occ, st);
        case PBG_ACCEL_RAYBVH: return bvh_occluded(s, o, d, valid, n, occ, st);
        case PBG_ACCEL_RAYHIERARCHY: return rh_occluded(s, o, d, valid, n, occ, st);
    }
    set_last_error("unknown accelerator kind");
    return PBG_ERR_INVALID_ARGUMENT;
}

// Copies the caller's host rays into the scene's work buffers.
// A device-usable address for caller memory, or nullptr: device and managed
// memory as is, pinned host memory through its mapping, and any host memory
// when the GPU reads the host's page tables directly (Grace-class hosts,
// where the coherent chip-to-chip link serves such reads at full rate).
static const void* device_view(int device, const void* p) {
    if (!p) return nullptr;
    // per device: 0 not probed yet, 1 no host page-table access, 2 access
    static std::atomic<int> ats[64];
    if (device >= 0 && device < 64 && ats[device].load() == 0) {
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
        ats[device].store(pageable && host_tables ? 2 : 1);
    }
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess) {
        if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
        if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    } else {
        cudaGetLastError();
    }
    return (device >= 0 && device < 64 && ats[device].load() == 2) ? p : nullptr;
}

// Caller SoA rows read in place (device-usable addresses) -> 16-byte records,
// the validity mask copied alongside.
__global__ void pack_rows_kernel(const float* __restrict__ ox, const float* __restrict__ oy,
                                 const float* __restrict__ oz, const float* __restrict__ dx,
                                 const float* __restrict__ dy, const float* __restrict__ dz,
                                 const float* __restrict__ mint, const float* __restrict__ maxt,
                                 const uint8_t* __restrict__ valid_in, int64_t n, float4* __restrict__ o,
                                 float4* __restrict__ d, uint8_t* __restrict__ valid_out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (valid_in) {  // an invalid ray's row entries are never read: skip them on the link
            const uint8_t v = valid_in[i];
            valid_out[i] = v;
            if (v == 0) {
                o[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                d[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                continue;
            }
        }
        o[i] = make_float4(ox[i], oy[i], oz[i], mint[i]);
        d[i] = make_float4(dx[i], dy[i], dz[i], maxt[i]);
    }
}

// The same gather in CTAs of 64 threads, four rays in flight per thread:
// small enough to sit beside a traversal kernel's resident CTAs (a 256-thread
// CTA does not fit beside five 256-thread CTAs of 48 registers), with enough
// loads in flight to keep the host link busy from one CTA per SM.
constexpr int kNarrowThreads = 64, kNarrowRays = 4;

__global__ void __launch_bounds__(kNarrowThreads)
    pack_rows_narrow_kernel(const float* __restrict__ ox, const float* __restrict__ oy,
                            const float* __restrict__ oz, const float* __restrict__ dx,
                            const float* __restrict__ dy, const float* __restrict__ dz,
                            const float* __restrict__ mint, const float* __restrict__ maxt,
                            const uint8_t* __restrict__ valid_in, int64_t n, float4* __restrict__ o,
                            float4* __restrict__ d, uint8_t* __restrict__ valid_out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; base < n; base += kNarrowRays * stride) {
        uint8_t v[kNarrowRays];
#pragma unroll
        for (int k = 0; k < kNarrowRays; ++k) {
            const int64_t i = base + k * stride;
            v[k] = i < n ? (valid_in ? valid_in[i] : (uint8_t)1) : (uint8_t)0;
        }
        float4 a[kNarrowRays], b[kNarrowRays];
#pragma unroll
        for (int k = 0; k < kNarrowRays; ++k) {
            const int64_t i = base + k * stride;
            a[k] = b[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (v[k]) {  // an invalid ray's row entries are never read
                a[k] = make_float4(ox[i], oy[i], oz[i], mint[i]);
                b[k] = make_float4(dx[i], dy[i], dz[i], maxt[i]);
            }
        }
#pragma unroll
        for (int k = 0; k < kNarrowRays; ++k) {
            const int64_t i = base + k * stride;
            if (i < n) {
                o[i] = a[k];
                d[i] = b[k];
                if (valid_in) valid_out[i] = v[k];
            }
        }
    }
}

// Results written in place to device-usable caller addresses.
__global__ void store_hits_kernel(const int32_t* __restrict__ prim, const float* __restrict__ t,
                                  const float* __restrict__ b1, const float* __restrict__ b2, int64_t n,
                                  int32_t* __restrict__ prim_out, float* __restrict__ t_out,
                                  float* __restrict__ b1_out, float* __restrict__ b2_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    prim_out[i] = prim[i];
    t_out[i] = t[i];
    b1_out[i] = b1[i];
    b2_out[i] = b2[i];
}

__global__ void store_bytes_kernel(const uint8_t* __restrict__ src, int64_t n, uint8_t* __restrict__ dst) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

static int stage_rays(pbg_scene* s, const pbg_rays* r, int64_t n, float4** o, float4** d,
                      uint8_t** valid) {
    Work& w = s->work;
    int rc;
    {  // read the caller's rows in place when the GPU can address them
        const float* rows[8] = {r->ox, r->oy, r->oz, r->dx, r->dy, r->dz, r->mint, r->maxt};
        const float* dv[8];
        bool direct = true;
        for (int k = 0; k < 8 && direct; ++k) direct = (dv[k] = (const float*)device_view(s->device, rows[k]));
        const uint8_t* vin = nullptr;
        if (direct && r->valid) direct = (vin = (const uint8_t*)device_view(s->device, r->valid)) != nullptr;
        if (direct) {
            if ((rc = ensure(w.ray_o, (size_t)n * sizeof(float4))) ||
                (rc = ensure(w.ray_d, (size_t)n * sizeof(float4))) ||
                (r->valid && (rc = ensure(w.valid, (size_t)n))))
                return rc;
            *o = (float4*)w.ray_o.ptr;
            *d = (float4*)w.ray_d.ptr;
            *valid = r->valid ? (uint8_t*)w.valid.ptr : nullptr;
            prof_begin(s, s->stream);
            pack_rows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(
                dv[0], dv[1], dv[2], dv[3], dv[4], dv[5], dv[6], dv[7], vin, n, *o, *d, *valid);
            prof_end(s, s->stream, kStageOther, 1);
            PBG_CUDA(cudaGetLastError());
            return PBG_OK;
        }
    }
    if ((rc = ensure(w.stage, (size_t)n * 8 * sizeof(float)))) return rc;
    if ((rc = ensure(w.ray_o, (size_t)n * sizeof(float4)))) return rc;
    if ((rc = ensure(w.ray_d, (size_t)n * sizeof(float4)))) return rc;
    float* stage = (float*)w.stage.ptr;
    const float* rows[8] = {r->ox, r->oy, r->oz, r->dx, r->dy, r->dz, r->mint, r->maxt};
    bool contiguous = true;
    for (int k = 1; k < 8; ++k)
        if (rows[k] != rows[0] + k * n) contiguous = false;
    if (contiguous) {
        PBG_CUDA(cudaMemcpyAsync(stage, rows[0], (size_t)n * 8 * sizeof(float),
                                 cudaMemcpyHostToDevice, s->stream));
    } else {
        for (int k = 0; k < 8; ++k)
            PBG_CUDA(cudaMemcpyAsync(stage + (size_t)k * n, rows[k], (size_t)n * sizeof(float),
                                     cudaMemcpyHostToDevice, s->stream));
    }
    *valid = nullptr;
    if (r->valid) {
        if ((rc = ensure(w.valid, (size_t)n))) return rc;
        PBG_CUDA(cudaMemcpyAsync(w.valid.ptr, r->valid, (size_t)n, cudaMemcpyHostToDevice,
                                 s->stream));
        *valid = (uint8_t*)w.valid.ptr;
    }
    *o = (float4*)w.ray_o.ptr;
    *d = (float4*)w.ray_d.ptr;
    return launch_pack_rays(s, stage, n, *o, *d, s->stream);
}

static bool is_pinned(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The high-priority stream (and its events) of the host-link copies.
static int ensure_io_stream(pbg_scene* s) {
    if (s->io_stream) return PBG_OK;
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    PBG_CUDA(cudaStreamCreateWithPriority(&s->io_stream, cudaStreamNonBlocking, hi));
    for (cudaEvent_t& e : s->io_events) PBG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return PBG_OK;
}

// Host-buffer nearest-hit calls of at least 2^21 rays on pinned memory run
// as two halves (of the declared ray image's rows, when there is one): the
// second half's rays cross the host link while the first half is traced,
// and the first half's hits cross back while the second is traced.  The
// copies run on the copy engines from a second stream, so they take no SMs
// from the traversal.  The host link moves about 210 GB/s each way, which
// for a 4 M-ray camera batch is 0.64 ms in and 0.35 ms out against about
// 0.9 ms of traversal.  *done = false: not applicable, nothing was started.
constexpr int kHostParts = 2;  // measured: 4 parts cost the rayhierarchy frame 2.6 % of e2e

static int intersect_two_halves(pbg_scene* s, const pbg_rays* r, int64_t n, pbg_hits* out,
                                bool* done) {
    *done = false;
    if (n < (int64_t(1) << 21)) return PBG_OK;
    const float* rows[8] = {r->ox, r->oy, r->oz, r->dx, r->dy, r->dz, r->mint, r->maxt};
    for (const float* q : rows)
        if (!is_pinned(q)) return PBG_OK;
    if (r->valid && !is_pinned(r->valid)) return PBG_OK;
    void* outs[4] = {out->prim, out->t, out->b1, out->b2};
    for (void* q : outs)
        if (!is_pinned(q)) return PBG_OK;
    // parts on whole image rows when a ray image of this size is declared
    constexpr int P = kHostParts;
    const bool image = s->image_w > 0 && n == s->image_w * s->image_h;
    if (image && (s->image_h % P) != 0) return PBG_OK;
    int64_t lo_of[P + 1];
    // without an image, boundaries on multiples of 4,096 rays (whole cache lines of the rows)
    for (int c = 0; c <= P; ++c)
        lo_of[c] = image ? (s->image_h / P) * c * s->image_w : c == P ? n : (n * c / P) & ~int64_t(4095);
    Work& w = s->work;
    int rc;
    if ((rc = ensure(w.stage, (size_t)n * 8 * sizeof(float))) ||
        (rc = ensure(w.ray_o, (size_t)n * sizeof(float4))) ||
        (rc = ensure(w.ray_d, (size_t)n * sizeof(float4))) ||
        (r->valid && (rc = ensure(w.valid, (size_t)n))) || (rc = ensure(w.prim, (size_t)n * 4)) ||
        (rc = ensure(w.t, (size_t)n * 4)) || (rc = ensure(w.b1, (size_t)n * 4)) ||
        (rc = ensure(w.b2, (size_t)n * 4)))
        return rc;
    if ((rc = ensure_io_stream(s))) return rc;
    float* stage = (float*)w.stage.ptr;
    uint8_t* vdev = r->valid ? (uint8_t*)w.valid.ptr : nullptr;
    for (int c = 0; c < P; ++c) {  // every part's rays in, in order
        const int64_t lo = lo_of[c], cnt = lo_of[c + 1] - lo_of[c];
        for (int k = 0; k < 8; ++k)
            PBG_CUDA(cudaMemcpyAsync(stage + (size_t)k * n + lo, rows[k] + lo, (size_t)cnt * 4,
                                     cudaMemcpyHostToDevice, s->io_stream));
        if (vdev)
            PBG_CUDA(cudaMemcpyAsync(vdev + lo, r->valid + lo, (size_t)cnt, cudaMemcpyHostToDevice,
                                     s->io_stream));
        PBG_CUDA(cudaEventRecord(s->io_events[c], s->io_stream));
    }
    const int64_t image_h = s->image_h;
    if (image) s->image_h = image_h / P;  // each part is a ray image of 1/P of the rows
    float4* o = (float4*)w.ray_o.ptr;
    float4* d = (float4*)w.ray_d.ptr;
    int32_t* prim = (int32_t*)w.prim.ptr;
    float *t = (float*)w.t.ptr, *b1 = (float*)w.b1.ptr, *b2 = (float*)w.b2.ptr;
    for (int c = 0; c < P && rc == PBG_OK; ++c) {
        const int64_t lo = lo_of[c], cnt = lo_of[c + 1] - lo_of[c];
        cudaStreamWaitEvent(s->stream, s->io_events[c], 0);
        const float* sr[8];
        for (int k = 0; k < 8; ++k) sr[k] = stage + (size_t)k * n + lo;
        prof_begin(s, s->stream);
        pack_rows_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s->stream>>>(
            sr[0], sr[1], sr[2], sr[3], sr[4], sr[5], sr[6], sr[7], vdev ? vdev + lo : nullptr, cnt, o + lo,
            d + lo, vdev ? vdev + lo : nullptr);
        prof_end(s, s->stream, kStageOther, 1);
        if (cudaGetLastError() != cudaSuccess) {
            rc = PBG_ERR_INTERNAL;
            break;
        }
        rc = run_nearest(s, o + lo, d + lo, vdev ? vdev + lo : nullptr, cnt, prim + lo, t + lo, b1 + lo,
                         b2 + lo, s->stream);
        if (rc) break;
        cudaEventRecord(s->io_events[P + c], s->stream);
        cudaStreamWaitEvent(s->io_stream, s->io_events[P + c], 0);
        const void* src[4] = {prim + lo, t + lo, b1 + lo, b2 + lo};
        for (int k = 0; k < 4; ++k)
            if (cudaMemcpyAsync((char*)outs[k] + lo * 4, src[k], (size_t)cnt * 4, cudaMemcpyDeviceToHost,
                                s->io_stream) != cudaSuccess)
                rc = PBG_ERR_INTERNAL;
    }
    s->image_h = image_h;
    const cudaError_t e = cudaStreamSynchronize(s->io_stream);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_status(e, "intersect_two_halves");
    *done = true;
    return check_device_status(s, s->stream);
}

void release_work(Work& w) {
    DeviceBuffer* all[] = {&w.ray_o, &w.ray_d, &w.ray_o2, &w.ray_d2, &w.valid, &w.prim,
                           &w.t, &w.b1, &w.b2, &w.occ, &w.keys, &w.stage, &w.perm,
                           &w.perm_tmp, &w.mkeys, &w.mkeys_tmp, &w.hist, &w.nodes,
                           &w.leafmask, &w.counters, &w.geo, &w.queue_a, &w.queue_b,
                           &w.qcount, &w.scan_sums, &w.pair_rank, &w.leafcnt, &w.origin_cache,
                           &w.osort_keys, &w.osort_perm, &w.reach,
                           &w.origin_valid};
    for (DeviceBuffer* b : all) release(*b);
    w.origin_sort_n = -1;
    w.origin_reused = false;
    w.origin_speculative = false;
    w.sorted_origins_ok = false;
}

// Host-buffer shadow calls of at least 2^21 rays whose rows and result the
// GPU addresses in place (pinned, or host page tables) run as two parts,
// each with its own work buffers and so its own kept origin order: the
// second part's rows cross the host link, read by a narrow gather kernel of
// one 64-thread CTA per SM on the high-priority stream, while the first part
// is traced, and the first part's results cross back the same way while the
// second part is traced.  Only valid rays' rows are read.  *done = false:
// not applicable, nothing was started.
constexpr int kShadowParts = 2;
// Share of the first part, whose rows cross the link with nothing to hide
// them behind: measured best of 40, 45 and 50 (a smaller first part leaves
// the second part's gather longer than the first part's traversal).
constexpr int kFirstPartPct = 50;

static int occluded_in_parts(pbg_scene* s, const pbg_rays* r, int64_t n, uint8_t* occ, bool* done) {
    *done = false;
    if (n < (int64_t(1) << 21)) return PBG_OK;
    const float* rows[8] = {r->ox, r->oy, r->oz, r->dx, r->dy, r->dz, r->mint, r->maxt};
    const float* dv[8];
    for (int k = 0; k < 8; ++k)
        if (!(dv[k] = (const float*)device_view(s->device, rows[k]))) return PBG_OK;
    const uint8_t* vin = nullptr;
    if (r->valid && !(vin = (const uint8_t*)device_view(s->device, r->valid))) return PBG_OK;
    uint8_t* po = (uint8_t*)device_view(s->device, occ);
    if (!po) return PBG_OK;
    constexpr int P = kShadowParts;
    static_assert(P == 2, "two work buffer sets");
    // the boundary on a multiple of 4,096 rays keeps both parts' host rows
    // and result bytes aligned to whole cache lines
    const int64_t lo_of[P + 1] = {0, (n * kFirstPartPct / 100) & ~int64_t(4095), n};
    Work* wp[P] = {&s->work, &s->alt};
    int rc;
    for (int c = 0; c < P; ++c) {
        const size_t cnt = (size_t)(lo_of[c + 1] - lo_of[c]);
        if ((rc = ensure(wp[c]->ray_o, cnt * sizeof(float4))) ||
            (rc = ensure(wp[c]->ray_d, cnt * sizeof(float4))) || (rc = ensure(wp[c]->occ, cnt)) ||
            (vin && (rc = ensure(wp[c]->valid, cnt))))
            return rc;
    }
    if ((rc = ensure_io_stream(s))) return rc;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    for (int c = 0; c < P; ++c) {  // every part's rows in, in order
        const int64_t lo = lo_of[c], cnt = lo_of[c + 1] - lo_of[c];
        Work& w = *wp[c];
        prof_begin(s, s->io_stream);
        if (c == 0) {
            pack_rows_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s->io_stream>>>(
                dv[0] + lo, dv[1] + lo, dv[2] + lo, dv[3] + lo, dv[4] + lo, dv[5] + lo, dv[6] + lo,
                dv[7] + lo, vin ? vin + lo : nullptr, cnt, (float4*)w.ray_o.ptr, (float4*)w.ray_d.ptr,
                vin ? (uint8_t*)w.valid.ptr : nullptr);
        } else {  // beside the first part's traversal: one narrow CTA per SM
            pack_rows_narrow_kernel<<<(unsigned)sms, kNarrowThreads, 0, s->io_stream>>>(
                dv[0] + lo, dv[1] + lo, dv[2] + lo, dv[3] + lo, dv[4] + lo, dv[5] + lo, dv[6] + lo,
                dv[7] + lo, vin ? vin + lo : nullptr, cnt, (float4*)w.ray_o.ptr, (float4*)w.ray_d.ptr,
                vin ? (uint8_t*)w.valid.ptr : nullptr);
        }
        prof_end(s, s->io_stream, kStageOther, 1);
        PBG_CUDA(cudaGetLastError());
        PBG_CUDA(cudaEventRecord(s->io_events[c], s->io_stream));
    }
    rc = PBG_OK;
    for (int c = 0; c < P && rc == PBG_OK; ++c) {
        const int64_t lo = lo_of[c], cnt = lo_of[c + 1] - lo_of[c];
        cudaStreamWaitEvent(s->stream, s->io_events[c], 0);
        Work& w = *wp[c];
        const float4* o = (const float4*)w.ray_o.ptr;
        const float4* d = (const float4*)w.ray_d.ptr;
        const uint8_t* v = vin ? (const uint8_t*)w.valid.ptr : nullptr;
        uint8_t* oc = (uint8_t*)w.occ.ptr;
        if (c > 0) std::swap(s->work, s->alt);  // the part's own buffers and kept order
        rc = run_occluded(s, o, d, v, cnt, oc, s->stream);
        if (c > 0) std::swap(s->work, s->alt);
        if (rc) break;
        if (c + 1 < P) {  // beside the next part's traversal: narrow CTAs on the copy stream
            cudaEventRecord(s->io_events[P + c], s->stream);
            cudaStreamWaitEvent(s->io_stream, s->io_events[P + c], 0);
            store_bytes_kernel<<<(unsigned)sms, kNarrowThreads, 0, s->io_stream>>>(oc, cnt, po + lo);
        } else {
            store_bytes_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s->stream>>>(oc, cnt, po + lo);
        }
        if (cudaGetLastError() != cudaSuccess) rc = PBG_ERR_INTERNAL;
    }
    const cudaError_t e = cudaStreamSynchronize(s->io_stream);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_status(e, "occluded_in_parts");
    *done = true;
    return check_device_status(s, s->stream);
}

static bool rays_ok(const pbg_rays* r) {
    return r && r->ox && r->oy && r->oz && r->dx && r->dy && r->dz && r->mint && r->maxt;
}

}  // namespace pbg

using namespace pbg;

extern "C" {

const char* pbg_version(void) { return "pbrt-gb300 1.0 (sm_103a)"; }

const char* pbg_status_string(int status) {
    switch (status) {
        case PBG_OK: return "ok";
        case PBG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PBG_ERR_CUDA: return "CUDA error";
        case PBG_ERR_OUT_OF_MEMORY: return "out of device memory";
        case PBG_ERR_DEVICE_TIMEOUT: return "bounded device wait expired";
        case PBG_ERR_NO_DEVICE: return "no CUDA device";
        case PBG_ERR_UNSUPPORTED: return "unsupported";
        case PBG_ERR_INTERNAL: return "internal error";
    }
    return "unknown status";
}

const char* pbg_last_error(void) { return g_last_error.c_str(); }

int pbg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // extern "C"

namespace pbg {

int build_bvh_device(pbg_scene* s, const float* tri9, int64_t ntri, int max_leaf, int32_t* order_dev,
                     cudaStream_t st);

// pbrt's TriangleMesh arrays -> the 9 floats (and 6 uvs) of each triangle.
__global__ void gather_mesh_kernel(const float* __restrict__ P, const int32_t* __restrict__ vi,
                                   const float* __restrict__ uv, int64_t ntri, int64_t nverts,
                                   float* __restrict__ tri9, float* __restrict__ uv6, int* __restrict__ bad) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntri) return;
    for (int k = 0; k < 3; ++k) {
        int32_t v = vi[3 * i + k];
        if (v < 0 || v >= nverts) {  // an index outside the vertex array: reported, read as vertex 0
            atomicAdd(bad, 1);
            v = 0;
        }
        for (int a = 0; a < 3; ++a) tri9[9 * i + 3 * k + a] = P[3 * (int64_t)v + a];
        if (uv6) {
            uv6[6 * i + 2 * k] = uv[2 * (int64_t)v];
            uv6[6 * i + 2 * k + 1] = uv[2 * (int64_t)v + 1];
        }
    }
}

// The scene's accelerator structures from triangles already in s->tri9 on
// the device: naive needs only the records; ray-bvh builds its tree on the
// device.  (rayhierarchy orders its records on the host; see scene_build.)
static int scene_build_device(pbg_scene* s) {
    const int64_t ntri = s->ntri;
    const size_t nt = (size_t)(ntri > 0 ? ntri : 1);
    int rc;
    if ((rc = ensure(s->tris, nt * sizeof(TriRec))) || (rc = ensure(s->tri_pos, nt * sizeof(int32_t)))) return rc;
    DeviceBuffer order;
    if (s->accel == PBG_ACCEL_RAYBVH) {
        if ((rc = ensure(order, nt * sizeof(int32_t)))) return rc;
        rc = build_bvh_device(s, (const float*)s->tri9.ptr, ntri, s->params.max_bvh_prim > 0 ? s->params.max_bvh_prim : 4,
                              (int32_t*)order.ptr, s->stream);
        if (rc) {
            release(order);
            return rc;
        }
    } else {
        // scene bounds for the naive scene (the device builder computes them for ray-bvh)
        std::vector<float> h((size_t)ntri * 9);
        if (ntri > 0) PBG_CUDA(cudaMemcpy(h.data(), s->tri9.ptr, h.size() * 4, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < ntri; ++i)
            for (int k = 0; k < 9; ++k) {
                const float v = h[9 * i + k];
                const int a = k % 3;
                if (i == 0 && k < 3) s->scene_lo[a] = s->scene_hi[a] = v;
                s->scene_lo[a] = v < s->scene_lo[a] ? v : s->scene_lo[a];
                s->scene_hi[a] = v > s->scene_hi[a] ? v : s->scene_hi[a];
            }
    }
    if (ntri > 0) {
        build_tris_kernel<<<(unsigned)((ntri + 255) / 256), 256, 0, s->stream>>>(
            (const float*)s->tri9.ptr, (const int32_t*)order.ptr, ntri, (TriRec*)s->tris.ptr, (int32_t*)s->tri_pos.ptr);
        s->counters.kernel_launches += 1;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    release(order);
    if (e != cudaSuccess) return cuda_status(e, "build_tris_kernel");
    return PBG_OK;
}

// The stream, status words and mailbox of a new scene.
static int scene_init(pbg_scene* s) {
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamCreate");
    int rc;
    if ((rc = ensure(s->err, 4 * sizeof(int)))) return rc;
    e = cudaHostAlloc((void**)&s->mbox_host, kMailboxWords * sizeof(int), cudaHostAllocMapped);
    if (e == cudaSuccess) memset(s->mbox_host, 0, kMailboxWords * sizeof(int));
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&s->mbox_dev, s->mbox_host, 0);
    if (e != cudaSuccess) return cuda_status(e, "cudaHostAlloc(status words)");
    if (cudaMemset(s->err.ptr, 0, 4 * sizeof(int)) != cudaSuccess)
        return cuda_status(cudaGetLastError(), "cudaMemset");
    return PBG_OK;
}

static int scene_args(const char* what, int64_t ntri, int32_t accel, pbg_scene** out) {
    if (!out) {
        set_last_error(std::string(what) + ": out is NULL");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (ntri < 0 || ntri > (int64_t)INT32_MAX / 2) {
        set_last_error(std::string(what) + ": bad triangle count");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (accel != PBG_ACCEL_NAIVE && accel != PBG_ACCEL_RAYHIERARCHY && accel != PBG_ACCEL_RAYBVH) {
        set_last_error(std::string(what) + ": unknown accelerator kind");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (pbg_device_count() == 0) {
        set_last_error(std::string(what) + ": no CUDA device");
        return PBG_ERR_NO_DEVICE;
    }
    return PBG_OK;
}

}  // namespace pbg

extern "C" {

int pbg_scene_create_mesh(const float* P, int64_t nverts, const int32_t* indices, int64_t ntri, const float* uv,
                          int32_t accel, const pbg_params* params, pbg_scene** out) {
    int rc = scene_args("pbg_scene_create_mesh", ntri, accel, out);
    if (rc) return rc;
    if (nverts < 0 || (ntri > 0 && (!P || !indices || nverts == 0))) {
        set_last_error("pbg_scene_create_mesh: bad vertex or index array");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (accel == PBG_ACCEL_RAYHIERARCHY) {  // its record order and spheres are built on the host
        std::vector<float> tri9((size_t)ntri * 9), uv6(uv ? (size_t)ntri * 6 : 0);
        for (int64_t i = 0; i < ntri; ++i)
            for (int k = 0; k < 3; ++k) {
                const int32_t v = indices[3 * i + k];
                if (v < 0 || v >= nverts) {
                    set_last_error("pbg_scene_create_mesh: vertex index out of range");
                    return PBG_ERR_INVALID_ARGUMENT;
                }
                for (int a = 0; a < 3; ++a) tri9[9 * i + 3 * k + a] = P[3 * (int64_t)v + a];
                if (uv) {
                    uv6[6 * i + 2 * k] = uv[2 * (int64_t)v];
                    uv6[6 * i + 2 * k + 1] = uv[2 * (int64_t)v + 1];
                }
            }
        return pbg_scene_create(tri9.data(), uv ? uv6.data() : nullptr, ntri, accel, params, out);
    }
    pbg_scene* s = new (std::nothrow) pbg_scene();
    if (!s) return PBG_ERR_OUT_OF_MEMORY;
    if (params) s->params = *params;
    s->device = s->params.device;
    s->accel = accel;
    s->ntri = ntri;
    auto fail = [&](int code) {
        pbg_scene_destroy(s);
        return code;
    };
    if ((rc = scene_init(s))) return fail(rc);
    const size_t nt = (size_t)(ntri > 0 ? ntri : 1);
    if ((rc = ensure(s->tri9, nt * 9 * sizeof(float)))) return fail(rc);
    if (uv && (rc = ensure(s->uv6, nt * 6 * sizeof(float)))) return fail(rc);
    if (ntri > 0) {
        DeviceBuffer dp, di, du;
        struct G {
            DeviceBuffer *a, *b, *c;
            ~G() { release(*a); release(*b); release(*c); }
        } g{&dp, &di, &du};
        if ((rc = ensure(dp, (size_t)nverts * 12)) || (rc = ensure(di, (size_t)ntri * 12)) ||
            (uv && (rc = ensure(du, (size_t)nverts * 8))))
            return fail(rc);
        cudaStream_t st = s->stream;
        cudaError_t e = cudaMemcpyAsync(dp.ptr, P, (size_t)nverts * 12, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(di.ptr, indices, (size_t)ntri * 12, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && uv) e = cudaMemcpyAsync(du.ptr, uv, (size_t)nverts * 8, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->err.ptr, 0, sizeof(int), st);
        if (e != cudaSuccess) return fail(cuda_status(e, "pbg_scene_create_mesh upload"));
        gather_mesh_kernel<<<(unsigned)((ntri + 255) / 256), 256, 0, st>>>(
            (const float*)dp.ptr, (const int32_t*)di.ptr, uv ? (const float*)du.ptr : nullptr, ntri, nverts,
            (float*)s->tri9.ptr, uv ? (float*)s->uv6.ptr : nullptr, (int*)s->err.ptr);
        s->counters.kernel_launches += 1;
        int bad = 0;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, s->err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail(cuda_status(e, "gather_mesh_kernel"));
        if (bad) {
            PBG_CUDA(cudaMemset(s->err.ptr, 0, sizeof(int)));
            set_last_error("pbg_scene_create_mesh: vertex index out of range");
            return fail(PBG_ERR_INVALID_ARGUMENT);
        }
    }
    if ((rc = scene_build_device(s))) return fail(rc);
    *out = s;
    return PBG_OK;
}

int pbg_scene_create(const float* tri9, const float* uv6, int64_t ntri, int32_t accel,
                     const pbg_params* params, pbg_scene** out) {
    int rc0 = scene_args("pbg_scene_create", ntri, accel, out);
    if (rc0) return rc0;
    if (ntri > 0 && !tri9) {
        set_last_error("pbg_scene_create: bad triangle array");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    pbg_scene* s = new (std::nothrow) pbg_scene();
    if (!s) return PBG_ERR_OUT_OF_MEMORY;
    if (params) s->params = *params;
    s->device = s->params.device;
    s->accel = accel;
    s->ntri = ntri;
    int rc = PBG_OK;
    auto fail = [&](int code) {
        pbg_scene_destroy(s);
        return code;
    };
    if (accel != PBG_ACCEL_RAYHIERARCHY && !(accel == PBG_ACCEL_RAYBVH && s->params.bvh_build == 1)) {
        // the triangles go to the device as they are; the rest is built there
        if ((rc = scene_init(s))) return fail(rc);
        const size_t nt = (size_t)(ntri > 0 ? ntri : 1);
        if ((rc = ensure(s->tri9, nt * 9 * sizeof(float)))) return fail(rc);
        if (ntri > 0) {
            cudaError_t e = cudaMemcpy(s->tri9.ptr, tri9, (size_t)ntri * 9 * sizeof(float), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return fail(cuda_status(e, "cudaMemcpy(triangles)"));
        }
        if ((rc = scene_build_device(s))) return fail(rc);
        if (uv6 && ntri > 0) {
            if ((rc = ensure(s->uv6, (size_t)ntri * 6 * sizeof(float)))) return fail(rc);
            cudaError_t e = cudaMemcpy(s->uv6.ptr, uv6, (size_t)ntri * 6 * sizeof(float), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return fail(cuda_status(e, "cudaMemcpy(uv)"));
        }
        *out = s;
        return PBG_OK;
    }
    // rayhierarchy (and ray-bvh with bvh_build = 1): record order built on the host
    if ((rc = scene_init(s))) return fail(rc);
    for (int64_t i = 0; i < ntri; ++i)
        for (int k = 0; k < 9; ++k) {
            float v = tri9[9 * i + k];
            if (i == 0 && k < 3) s->scene_lo[k] = s->scene_hi[k] = v;
            int a = k % 3;
            s->scene_lo[a] = v < s->scene_lo[a] ? v : s->scene_lo[a];
            s->scene_hi[a] = v > s->scene_hi[a] ? v : s->scene_hi[a];
        }
    HostBvh hb;
    std::vector<int32_t> morder;
    const int32_t* order = nullptr;
    if (accel == PBG_ACCEL_RAYHIERARCHY) {
        cluster_triangle_order(tri9, ntri, &morder);
        order = morder.empty() ? nullptr : morder.data();
    }
    if (accel == PBG_ACCEL_RAYBVH) {
        build_bvh(tri9, ntri, s->params.max_bvh_prim > 0 ? s->params.max_bvh_prim : 4, &hb);
        order = hb.order.empty() ? nullptr : hb.order.data();
        if ((rc = ensure(s->bvh, hb.nodes.size() * sizeof(BvhNode)))) return fail(rc);
        cudaError_t e = cudaMemcpy(s->bvh.ptr, hb.nodes.data(), hb.nodes.size() * sizeof(BvhNode),
                                   cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(cuda_status(e, "cudaMemcpy(bvh)"));
        s->bvh_nodes = (int64_t)hb.nodes.size();
        s->bvh_depth = hb.max_depth;
        s->unculled = hb.unculled;
        s->counters.bvh_nodes = (uint64_t)hb.nodes.size();
        s->host_nodes = hb.nodes;
        s->host_order = hb.order;
    }
    if ((rc = upload_triangles(s, tri9, order))) return fail(rc);
    if (uv6 && ntri > 0) {
        if ((rc = ensure(s->uv6, (size_t)ntri * 6 * sizeof(float)))) return fail(rc);
        cudaError_t e = cudaMemcpy(s->uv6.ptr, uv6, (size_t)ntri * 6 * sizeof(float),
                                   cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(cuda_status(e, "cudaMemcpy(uv)"));
    }
    *out = s;
    return PBG_OK;
}

void pbg_scene_destroy(pbg_scene* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    prof_collect(s);
    for (cudaEvent_t e : s->prof.pool) cudaEventDestroy(e);
    s->prof.pool.clear();
    release(s->tris);
    release(s->tri9);
    release(s->uv6);
    release(s->bvh);
    release(s->wide);
    release(s->tris_wide);
    release(s->spheres);
    release(s->clusters);
    release(s->tri_pos);
    release(s->err);
    release(s->workc);
    if (s->learn) {
        learn_free(s->learn);
        s->learn = nullptr;
    }
    release_work(s->work);
    release_work(s->alt);
    render_free(s);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->io_stream) {
        cudaStreamDestroy(s->io_stream);
        for (cudaEvent_t e : s->io_events)
            if (e) cudaEventDestroy(e);
    }
    if (s->mbox_host) cudaFreeHost(s->mbox_host);
    delete s;
}

int pbg_max_rays_per_call(const pbg_scene* s, int64_t* out) {
    if (!s || !out) return PBG_ERR_INVALID_ARGUMENT;
    // The reference's cap (naive.cpp:141) keeps its task tiling; the device
    // path itself has no per-call limit below 2^31 rays.
    *out = 409600;
    return PBG_OK;
}

// Device rays are read as float4: views that are not 16-byte aligned (a
// sliced tensor, an odd offset) are refused instead of faulting the GPU.
static bool rays_aligned(const float* o4, const float* d4) {
    return (((uintptr_t)o4 | (uintptr_t)d4) & 15u) == 0;
}

int pbg_intersect_device(pbg_scene* s, const float* o4, const float* d4, const uint8_t* valid,
                         int64_t n, int32_t* prim, float* t, float* b1, float* b2, void* stream) {
    if (!s || n < 0 || (n > 0 && (!o4 || !d4 || !prim || !t || !b1 || !b2)) || !rays_aligned(o4, d4)) {
        set_last_error("pbg_intersect_device: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (n > (int64_t)INT32_MAX) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    int rc = run_nearest(s, (const float4*)o4, (const float4*)d4, valid, n, prim, t, b1, b2, st);
    if (rc == PBG_OK) {
        s->counters.rays_nearest += (uint64_t)n;
        s->counters.calls++;
    }
    return rc;
}

int pbg_occluded_device(pbg_scene* s, const float* o4, const float* d4, const uint8_t* valid,
                        int64_t n, uint8_t* occ, void* stream) {
    if (!s || n < 0 || (n > 0 && (!o4 || !d4 || !occ)) || !rays_aligned(o4, d4)) {
        set_last_error("pbg_occluded_device: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (n > (int64_t)INT32_MAX) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    int rc = run_occluded(s, (const float4*)o4, (const float4*)d4, valid, n, occ, st);
    if (rc == PBG_OK) {
        s->counters.rays_occluded += (uint64_t)n;
        s->counters.calls++;
    }
    return rc;
}

int pbg_clusters_of_device(pbg_scene* s, const int32_t* prim, int64_t n, uint16_t* cluster, void* stream) {
    if (!s || n < 0 || (n > 0 && (!prim || !cluster))) {
        set_last_error("pbg_clusters_of_device: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(s->device);
    return clusters_of(s, prim, n, cluster, stream ? (cudaStream_t)stream : s->stream);
}

int pbg_intersect_hinted_device(pbg_scene* s, const float* o4, const float* d4, const uint8_t* valid, int64_t n,
                                const uint16_t* hint, int32_t* prim, float* t, float* b1, float* b2,
                                void* stream) {
    if (!s || n < 0 || n > (int64_t)INT32_MAX || (n > 0 && (!o4 || !d4 || !prim || !t || !b1 || !b2)) ||
        !rays_aligned(o4, d4)) {
        set_last_error("pbg_intersect_hinted_device: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (s->accel != PBG_ACCEL_RAYBVH) {
        set_last_error("pbg_intersect_hinted_device: cluster hints need Accelerator \"ray-bvh\"");
        return PBG_ERR_UNSUPPORTED;
    }
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    int rc = bvh_nearest_hinted(s, (const float4*)o4, (const float4*)d4, valid, n, hint, prim, t, b1, b2, st);
    if (rc == PBG_OK) {
        s->counters.rays_nearest += (uint64_t)n;
        s->counters.calls++;
    }
    return rc;
}

int pbg_occluded_hinted_device(pbg_scene* s, const float* o4, const float* d4, const uint8_t* valid, int64_t n,
                               const uint16_t* hint, uint8_t* occ, int32_t* occluders, void* stream) {
    if (!s || n < 0 || n > (int64_t)INT32_MAX || (n > 0 && (!o4 || !d4 || !occ)) || !rays_aligned(o4, d4)) {
        set_last_error("pbg_occluded_hinted_device: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (s->accel != PBG_ACCEL_RAYBVH) {
        set_last_error("pbg_occluded_hinted_device: cluster hints need Accelerator \"ray-bvh\"");
        return PBG_ERR_UNSUPPORTED;
    }
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    int rc = bvh_occluded_hinted(s, (const float4*)o4, (const float4*)d4, valid, n, hint, occ, occluders, st);
    if (rc == PBG_OK) {
        s->counters.rays_occluded += (uint64_t)n;
        s->counters.calls++;
    }
    return rc;
}

// Marks a host-buffer call for its duration (ray-bvh runs its packet walk
// in the caller's order there, see bvh_launch).
struct HostCall {
    pbg_scene* s;
    explicit HostCall(pbg_scene* sc) : s(sc) { s->host_call = true; }
    ~HostCall() { s->host_call = false; }
};

int pbg_intersect(pbg_scene* s, const pbg_rays* r, int64_t n, pbg_hits* out) {
    if (!s || n < 0 || (n > 0 && (!rays_ok(r) || !out || !out->prim || !out->t || !out->b1 ||
                                  !out->b2))) {
        set_last_error("pbg_intersect: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PBG_OK;
    cudaSetDevice(s->device);
    HostCall host_call(s);
    bool done = false;
    int rc = intersect_two_halves(s, r, n, out, &done);
    if (rc) return rc;
    if (done) {
        s->counters.rays_nearest += (uint64_t)n;
        s->counters.calls++;
        return PBG_OK;
    }
    float4 *o, *d;
    uint8_t* valid;
    rc = stage_rays(s, r, n, &o, &d, &valid);
    if (rc) return rc;
    Work& w = s->work;
    if ((rc = ensure(w.prim, (size_t)n * 4)) || (rc = ensure(w.t, (size_t)n * 4)) ||
        (rc = ensure(w.b1, (size_t)n * 4)) || (rc = ensure(w.b2, (size_t)n * 4)))
        return rc;
    rc = run_nearest(s, o, d, valid, n, (int32_t*)w.prim.ptr, (float*)w.t.ptr, (float*)w.b1.ptr,
                     (float*)w.b2.ptr, s->stream);
    if (rc) return rc;
    int32_t* pp = (int32_t*)device_view(s->device, out->prim);
    float* pt = (float*)device_view(s->device, out->t);
    float* p1 = (float*)device_view(s->device, out->b1);
    float* p2 = (float*)device_view(s->device, out->b2);
    if (pp && pt && p1 && p2) {
        store_hits_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(
            (const int32_t*)w.prim.ptr, (const float*)w.t.ptr, (const float*)w.b1.ptr,
            (const float*)w.b2.ptr, n, pp, pt, p1, p2);
        PBG_CUDA(cudaGetLastError());
    } else {
        PBG_CUDA(cudaMemcpyAsync(out->prim, w.prim.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream));
        PBG_CUDA(cudaMemcpyAsync(out->t, w.t.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream));
        PBG_CUDA(cudaMemcpyAsync(out->b1, w.b1.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream));
        PBG_CUDA(cudaMemcpyAsync(out->b2, w.b2.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream));
    }
    rc = check_device_status(s, s->stream);
    if (rc) return rc;
    s->counters.rays_nearest += (uint64_t)n;
    s->counters.calls++;
    return PBG_OK;
}

int pbg_occluded(pbg_scene* s, const pbg_rays* r, int64_t n, uint8_t* occ) {
    if (!s || n < 0 || (n > 0 && (!rays_ok(r) || !occ))) {
        set_last_error("pbg_occluded: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PBG_OK;
    cudaSetDevice(s->device);
    HostCall host_call(s);
    bool done = false;
    int rc = occluded_in_parts(s, r, n, occ, &done);
    if (rc) return rc;
    if (done) {
        s->counters.rays_occluded += (uint64_t)n;
        s->counters.calls++;
        return PBG_OK;
    }
    float4 *o, *d;
    uint8_t* valid;
    rc = stage_rays(s, r, n, &o, &d, &valid);
    if (rc) return rc;
    Work& w = s->work;
    if ((rc = ensure(w.occ, (size_t)n))) return rc;
    rc = run_occluded(s, o, d, valid, n, (uint8_t*)w.occ.ptr, s->stream);
    if (rc) return rc;
    if (uint8_t* po = (uint8_t*)device_view(s->device, occ)) {
        store_bytes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>((const uint8_t*)w.occ.ptr, n, po);
        PBG_CUDA(cudaGetLastError());
    } else {
        PBG_CUDA(cudaMemcpyAsync(occ, w.occ.ptr, (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    }
    rc = check_device_status(s, s->stream);
    if (rc) return rc;
    s->counters.rays_occluded += (uint64_t)n;
    s->counters.calls++;
    return PBG_OK;
}

int pbg_hit_geometry_device(pbg_scene* s, const float* o4, const float* d4, const int32_t* prim,
                            const float* t, const float* b1, const float* b2, int64_t n,
                            float* out14, void* stream) {
    if (!s || n < 0 || (n > 0 && (!o4 || !d4 || !prim || !t || !b1 || !b2 || !out14)) || !rays_aligned(o4, d4))
        return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    return hit_geometry(s, (const float4*)o4, (const float4*)d4, prim, t, b1, b2, n, out14, st);
}

int pbg_hit_geometry(pbg_scene* s, const pbg_rays* r, const pbg_hits* h, int64_t n,
                     float* out14) {
    if (!s || n < 0 || (n > 0 && (!rays_ok(r) || !h || !h->prim || !h->t || !h->b1 || !h->b2 ||
                                  !out14))) {
        set_last_error("pbg_hit_geometry: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PBG_OK;
    cudaSetDevice(s->device);
    float4 *o, *d;
    uint8_t* valid;
    int rc = stage_rays(s, r, n, &o, &d, &valid);
    if (rc) return rc;
    Work& w = s->work;
    if ((rc = ensure(w.prim, (size_t)n * 4)) || (rc = ensure(w.t, (size_t)n * 4)) ||
        (rc = ensure(w.b1, (size_t)n * 4)) || (rc = ensure(w.b2, (size_t)n * 4)) ||
        (rc = ensure(w.geo, (size_t)n * 14 * 4)))
        return rc;
    PBG_CUDA(cudaMemcpyAsync(w.prim.ptr, h->prim, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
    PBG_CUDA(cudaMemcpyAsync(w.t.ptr, h->t, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
    PBG_CUDA(cudaMemcpyAsync(w.b1.ptr, h->b1, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
    PBG_CUDA(cudaMemcpyAsync(w.b2.ptr, h->b2, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
    rc = hit_geometry(s, o, d, (const int32_t*)w.prim.ptr, (const float*)w.t.ptr,
                      (const float*)w.b1.ptr, (const float*)w.b2.ptr, n, (float*)w.geo.ptr,
                      s->stream);
    if (rc) return rc;
    PBG_CUDA(cudaMemcpyAsync(out14, w.geo.ptr, (size_t)n * 14 * 4, cudaMemcpyDeviceToHost, s->stream));
    PBG_CUDA(cudaStreamSynchronize(s->stream));
    return PBG_OK;
}

int pbg_stats(pbg_scene* s, pbg_counters* out) {
    if (!s || !out) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    prof_collect(s);
    *out = s->counters;
    return PBG_OK;
}

int pbg_preprocess(pbg_scene* s, int64_t width, int64_t height) {
    if (!s || width < 0 || height < 0 || (width > 0) != (height > 0) || width > (1 << 15) ||
        height > (1 << 15)) {
        set_last_error("pbg_preprocess: bad ray-image size (at most 32768 x 32768)");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    s->image_w = width;
    s->image_h = height;
    return PBG_OK;
}

int pbg_profile(pbg_scene* s, int on) {
    if (!s) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    prof_collect(s);
    s->prof.on = on != 0;
    s->prof.level = on;
    for (int k = 0; k < 4; ++k) {
        s->counters.stage_ms[k] = 0.0;
        s->counters.timed_launches[k] = 0;
    }
    for (int k = 0; k < 6; ++k) s->counters.work[k] = 0;
    if (on >= 2) {
        int rc = ensure(s->workc, 8 * sizeof(unsigned long long));
        if (rc) return rc;
        PBG_CUDA(cudaMemset(s->workc.ptr, 0, 8 * sizeof(unsigned long long)));
    }
    return PBG_OK;
}

}  // extern "C"
