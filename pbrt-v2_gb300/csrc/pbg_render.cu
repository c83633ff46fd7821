// pbg_render.cu -- the breadth-first renderer as a device wavefront.
//
// Reference: renderers/breadth-first.cpp:18-228 generates every camera ray
// of a task tile, calls the batch Li of the surface integrator, which shades
// on the host and sends shadow rays (core/integrator.cpp:73-455) and bounce
// rays (integrators/path.cpp:43-157) back as batches; rays that die keep
// their slot.  Here the whole image is one batch and every stage runs on the
// device:
//
//   raygen     camera rays from the caller's RasterToCamera / CameraToWorld
//              (cameras/perspective.cpp GenerateRayDifferential), stratified
//              image samples (samplers/stratified.cpp), scanline order with
//              spp consecutive samples (the breadth-first ray image);
//   trace      the scene's accelerator (pbg_*_device) on the live queue;
//   shade      Lambertian BSDF (core/reflection.cpp:165), light sampling
//              (lights/point.cpp; lights/diffuse.cpp over scene triangles as
//              ShapeSet samples them, core/light.cpp:137-165; a
//              parallelogram emitter), the batch integrators' EstimateDirect
//              (core/integrator.cpp:212-298 for path, :358-455 for
//              directlighting, each with its own operation order), emission
//              at camera hits on emitting triangles, one shadow slot per
//              light sample and one bounce slot per path;
//   compact    slots -> dense queues, order-preserving: per-warp ballots give
//              ranks inside a block, a block scan gives block offsets;
//   resolve    unoccluded shadow contributions added per sample in light
//              sample order (deterministic, no float atomics);
//   film       per pixel, samples in order, through XYZ as ImageFilm does
//              (film/image.cpp AddSample / WriteImage), box filter; samples
//              whose radiance breadthFirst::Li would reject (NaN, negative or
//              infinite luminance) count as black.
//
// Random numbers: by default a counter-based hash of (seed, sample,
// dimension), identical on every run and in the oracle's restatement.  With
// a sample stream (pbg_render_stream) the values are the reference's own:
// the caller passes one task's samples as pbrt's StratifiedSampler drew them
// and the continuation of the task's RNG, which the renderer consumes in
// the order the batch integrators do -- path tracing below bounce 3 reads
// the sample arrays (integrators/path.cpp:31-38), from bounce 3 on
// UniformSampleOneLight draws 7 values for every ray of the task, then each
// ray that hit draws its BSDF sample (3) and, after bounce 3, its Russian
// roulette value (1), in ray order (core/integrator.cpp:142-165,
// integrators/path.cpp:104-124).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pbg_dg.cuh"
#include "pbg_internal.h"
#include "pbg_learn.h"

namespace pbg {

constexpr float kInvPi = 0.31830988618379067154f;

// splitmix64 finalizer (a published 64-bit mixing function)
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform float in [0, 1) for (seed, sample, dim).
__device__ __forceinline__ float rnd(uint64_t seed, uint64_t sample, uint32_t dim) {
    const uint64_t h = mix64(seed ^ mix64(sample * 0x100000001B3ull + dim));
    return (float)(h >> 40) * 0x1p-24f;
}

// Sample dimensions: 0-1 image, then 16 per bounce: light samples from 0,
// Russian roulette at 13, BSDF sample at 14-15.  The light-sample
// components of triangle emitters and the light choice of the path
// integrator use a second family from 512.
__device__ __forceinline__ uint32_t dim_of(int bounce, int k) { return 2u + 16u * (uint32_t)bounce + (uint32_t)k; }
__device__ __forceinline__ uint32_t dim_extra(int bounce, int k) { return 512u + 16u * (uint32_t)bounce + (uint32_t)k; }
constexpr int kDimRR = 13, kDimBsdf = 14;

// sin and cos in float from the Cephes single-precision polynomials
// (S. Moshier, Cephes Math Library, sinf.c/cosf.c coefficients) after a
// two-constant Cody-Waite reduction by pi/2, every operation correctly
// rounded and unfused, so the oracle's C restatement gives identical bits.
__device__ __forceinline__ void own_sincos(float a, float* s, float* c) {
    const float jf = rintf(__fmul_rn(a, 0.636619772367581343f));
    const int j = (int)jf;
    const float r = __fsub_rn(__fsub_rn(a, __fmul_rn(jf, 1.5703125f)), __fmul_rn(jf, 4.83826794897e-4f));
    const float z = __fmul_rn(r, r);
    const float sp = __fadd_rn(__fmul_rn(__fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(__fmul_rn(-1.9515295891e-4f, z),
                                                                                    8.3321608736e-3f), z),
                                                               1.6666654611e-1f), z), r), r);
    const float cp = __fadd_rn(__fsub_rn(__fmul_rn(__fmul_rn(__fadd_rn(__fmul_rn(__fsub_rn(__fmul_rn(2.443315711809948e-5f, z),
                                                                                              1.388731625493765e-3f), z),
                                                                          4.166664568298827e-2f), z), z),
                                         __fmul_rn(0.5f, z)), 1.f);
    switch (j & 3) {
        case 0: *s = sp; *c = cp; break;
        case 1: *s = cp; *c = -sp; break;
        case 2: *s = -sp; *c = -cp; break;
        default: *s = -cp; *c = sp; break;
    }
}

struct DevLight {
    int type, nsamples;
    float pos[3], I[3];
    float q0[3], e1[3], e3[3], n[3], area, L[3];
    int first, ntri;  // triangle emitter: scene triangles [first, first + ntri)
    int tab;          // ... its areas, CDF and total area in the light table
};

struct RenderConst {
    float r2c[16], c2w[16];
    int xres, yres, spp_x, spp_y, spp, jitter, max_depth, integrator;
    uint64_t seed;
    float albedo[3];
    int nlights;
    DevLight lights[4];
    int stream;           // 1: sample values from the caller's stream
    const float* ltab;    // triangle emitters: areas[ntri], cdf[ntri + 1], sum
};

// The caller's sample stream on the device (see pbg_sample_stream).
struct StreamArgs {
    const float* img;        // [count][2] raster position
    const float* dims;       // [count][ndims]
    const float* rng;        // the task RNG's draws after the sampler's
    int64_t count, nrng;
    int ndims;
    int64_t rng_base;        // path, bounces >= 3: this bounce's first draw
    const int32_t* hit_rank; // ... and each queue entry's rank among its hits
};

__global__ void raygen_kernel(RenderConst rc, StreamArgs sa, int64_t n, float4* __restrict__ o4,
                              float4* __restrict__ d4, int32_t* __restrict__ qidx, float* __restrict__ L,
                              float* __restrict__ beta) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float ix, iy;
    if (rc.stream) {
        ix = sa.img[2 * s];
        iy = sa.img[2 * s + 1];
    } else {
        const int64_t pix = s / rc.spp;
        const int k = (int)(s % rc.spp);
        const int px = (int)(pix % rc.xres), py = (int)(pix / rc.xres);
        const int sx = k % rc.spp_x, sy = k / rc.spp_x;
        const float jx = rc.jitter ? rnd(rc.seed, (uint64_t)s, 0) : 0.5f;
        const float jy = rc.jitter ? rnd(rc.seed, (uint64_t)s, 1) : 0.5f;
        // (x + jx) * dx + xPos (samplers/stratified.cpp, StratifiedSample2D)
        ix = __fadd_rn(__fmul_rn(__fadd_rn((float)sx, jx), __frcp_rn((float)rc.spp_x)), (float)px);
        iy = __fadd_rn(__fmul_rn(__fadd_rn((float)sy, jy), __frcp_rn((float)rc.spp_y)), (float)py);
    }
    const V3 pc = xform_point(rc.r2c, v3(ix, iy, 0.f));
    const V3 dir = vnormalize(pc);
    const V3 o = xform_point(rc.c2w, v3(0.f, 0.f, 0.f));
    const V3 d = xform_vector(rc.c2w, dir);
    o4[s] = make_float4(o.x, o.y, o.z, 0.f);
    d4[s] = make_float4(d.x, d.y, d.z, INFINITY);
    qidx[s] = (int32_t)s;
    L[3 * s] = L[3 * s + 1] = L[3 * s + 2] = 0.f;
    beta[3 * s] = beta[3 * s + 1] = beta[3 * s + 2] = 1.f;
}

// Shading frame of pbrt's BSDF: nn, sn = Normalize(dpdu), tn = Cross(nn, sn).
struct Frame {
    V3 nn, sn, tn;
    __device__ V3 to_local(V3 v) const { return v3(vdot(v, sn), vdot(v, tn), vdot(v, nn)); }
    __device__ V3 to_world(V3 v) const {
        return v3(__fadd_rn(__fadd_rn(__fmul_rn(sn.x, v.x), __fmul_rn(tn.x, v.y)), __fmul_rn(nn.x, v.z)),
                  __fadd_rn(__fadd_rn(__fmul_rn(sn.y, v.x), __fmul_rn(tn.y, v.y)), __fmul_rn(nn.y, v.z)),
                  __fadd_rn(__fadd_rn(__fmul_rn(sn.z, v.x), __fmul_rn(tn.z, v.y)), __fmul_rn(nn.z, v.z)));
    }
};

__device__ __forceinline__ V3 tri_vertex(const float* v9, int k) { return v3(v9[3 * k], v9[3 * k + 1], v9[3 * k + 2]); }

// The scene triangle of an emitter's i-th ShapeSet shape: the ShapeSet
// constructor refines the mesh through a stack (todo.back(),
// core/light.cpp:106-118), so the mesh's triangles come out last first.
__device__ __forceinline__ int64_t shape_tri(int first, int n, int i) { return (int64_t)first + n - 1 - i; }

// Triangle::Intersect of one emitter triangle (shapes/trianglemesh.cpp:119-190):
// pbrt's exact test, and the hit's geometric normal.
__device__ bool emitter_hit(const float* v9, const float* uv6, V3 o, V3 d, float mint, float* t, V3* nn) {
    const V3 p1 = tri_vertex(v9, 0), e1 = vsub(tri_vertex(v9, 1), p1), e2 = vsub(tri_vertex(v9, 2), p1);
    float tt, b1, b2;
    if (!pbg_exact(p1.x, p1.y, p1.z, e1.x, e1.y, e1.z, e2.x, e2.y, e2.z, o.x, o.y, o.z, d.x, d.y, d.z, mint,
                   INFINITY, &tt, &b1, &b2))
        return false;
    *t = tt;
    *nn = hit_dg(v9, uv6, o, d, tt, b1, b2).nn;
    return true;
}

// DiffuseAreaLight::Sample_L over scene triangles (lights/diffuse.cpp:61-73):
// ShapeSet::Sample picks a triangle by its area CDF and a point on it
// (Triangle::Sample, UniformSampleTriangle), re-intersects the ray from p
// towards it with every triangle of the set (the last one hit gives the
// point and its normal), ShapeSet::Pdf sums each triangle's solid-angle pdf
// weighted by its area (core/light.cpp:137-165, core/shape.cpp:78-91).
__device__ void sample_emitter(const DevLight& lt, const float* ltab, const float* tri9, const float* uv6, V3 p,
                               float u0, float u1, float comp, V3* wi, V3* Li, float* pdf, V3* target) {
    const int n = lt.ntri;
    const float* areas = ltab + lt.tab;
    const float* cdf = areas + n;
    const float sum_area = cdf[n + 1];
    int k = 0;  // upper_bound: first CDF entry above comp
    while (k < n + 1 && !(cdf[k] > comp)) ++k;
    const int sn = k > 0 ? k - 1 : 0;
    const float* v = tri9 + 9 * shape_tri(lt.first, n, sn);
    const float su1 = __fsqrt_rn(u0);
    const float b1 = __fsub_rn(1.f, su1), b2 = __fmul_rn(u1, su1);
    const float b0 = __fsub_rn(__fsub_rn(1.f, b1), b2);
    const V3 p1 = tri_vertex(v, 0), p2 = tri_vertex(v, 1), p3 = tri_vertex(v, 2);
    const V3 pt = vadd(vadd(vmul(p1, b1), vmul(p2, b2)), vmul(p3, b0));
    V3 ns = vnormalize(vcross(vsub(p2, p1), vsub(p3, p1)));
    const V3 dir = vsub(pt, p);
    float thit = 1.f;
    for (int i = 0; i < n; ++i) {
        const int64_t tr = shape_tri(lt.first, n, i);
        float t;
        V3 nn;
        if (emitter_hit(tri9 + 9 * tr, uv6 ? uv6 + 6 * tr : nullptr, p, dir, 1e-3f, &t, &nn)) {
            thit = t;
            ns = nn;
        }
    }
    const V3 ps = vadd(p, vmul(dir, thit));
    *target = ps;
    *wi = vnormalize(vsub(ps, p));
    float acc = 0.f;
    for (int i = 0; i < n; ++i) {
        const int64_t tr = shape_tri(lt.first, n, i);
        float t, pi = 0.f;
        V3 nn;
        if (emitter_hit(tri9 + 9 * tr, uv6 ? uv6 + 6 * tr : nullptr, p, *wi, 1e-3f, &t, &nn)) {
            const V3 dv = vsub(p, vadd(p, vmul(*wi, t)));
            pi = __fdiv_rn(vdot(dv, dv), __fmul_rn(fabsf(vdot(nn, vneg(*wi))), areas[i]));
            if (isinf(pi)) pi = 0.f;
        }
        acc = __fadd_rn(acc, __fmul_rn(areas[i], pi));
    }
    *pdf = __fdiv_rn(acc, sum_area);
    *Li = vdot(ns, vneg(*wi)) > 0.f ? v3(lt.L[0], lt.L[1], lt.L[2]) : v3(0.f, 0.f, 0.f);
}

// Light sample (u0, u1, comp) of light lt at p: wi, radiance, pdf and the
// shadow segment (VisibilityTester::SetSegment, core/light.h:79-84).
__device__ __forceinline__ bool sample_light(const RenderConst& rc, const DevLight& lt, const float* tri9,
                                             const float* uv6, V3 p, float eps, float u1, float u2, float comp,
                                             V3* wi, V3* Li, float* pdf, float4* so, float4* sd) {
    V3 target;
    float eps2;
    if (lt.type == PBG_LIGHT_POINT) {
        target = v3(lt.pos[0], lt.pos[1], lt.pos[2]);
        *wi = vnormalize(vsub(target, p));
        *pdf = 1.f;
        const V3 dv = vsub(target, p);
        const float d2 = vdot(dv, dv);
        *Li = v3(__fdiv_rn(lt.I[0], d2), __fdiv_rn(lt.I[1], d2), __fdiv_rn(lt.I[2], d2));
        eps2 = 0.f;
    } else if (lt.type == PBG_LIGHT_MESH) {
        sample_emitter(lt, rc.ltab, tri9, uv6, p, u1, u2, comp, wi, Li, pdf, &target);
        eps2 = 1e-3f;
    } else {
        const V3 q0 = v3(lt.q0[0], lt.q0[1], lt.q0[2]);
        target = vadd(vadd(q0, vmul(v3(lt.e1[0], lt.e1[1], lt.e1[2]), u1)),
                      vmul(v3(lt.e3[0], lt.e3[1], lt.e3[2]), u2));
        const V3 dv = vsub(target, p);
        *wi = vnormalize(dv);
        const float d2 = vdot(dv, dv);
        const float cosl = -vdot(v3(lt.n[0], lt.n[1], lt.n[2]), *wi);
        if (!(cosl > 0.f) || !(d2 > 0.f)) return false;
        *pdf = __fdiv_rn(d2, __fmul_rn(cosl, lt.area));
        *Li = v3(lt.L[0], lt.L[1], lt.L[2]);
        eps2 = 1e-3f;
    }
    const float dist = vlen(vsub(p, target));
    const V3 dn = vmul(vsub(target, p), __frcp_rn(dist));
    *so = make_float4(p.x, p.y, p.z, eps);
    *sd = make_float4(dn.x, dn.y, dn.z, __fmul_rn(dist, __fsub_rn(1.f, eps2)));
    return true;
}

// Sample values of one vertex: the hash stream, or the caller's stream in
// the layout of pbg_sample_stream.
struct Draws {
    const RenderConst& rc;
    const StreamArgs& sa;
    int64_t s, j;
    int bounce;
    // light sample m of a directlighting vertex (hash: light-local index q)
    __device__ void direct_light(int m, int q, float* u0, float* u1, float* comp) const {
        if (rc.stream) {
            const float* v = sa.dims + s * sa.ndims + 6 * m;
            *u0 = v[0];
            *u1 = v[1];
            *comp = v[2];
        } else {
            *u0 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, 2 * q));
            *u1 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, 2 * q) + 1);
            *comp = rnd(rc.seed, (uint64_t)s, dim_extra(bounce, m));
        }
    }
    // the path integrator's light choice and light sample at this bounce
    __device__ void path_light(float* lnum, float* u0, float* u1, float* comp) const {
        if (!rc.stream) {
            *lnum = rnd(rc.seed, (uint64_t)s, dim_extra(bounce, 15));
            *u0 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, 0));
            *u1 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, 1));
            *comp = rnd(rc.seed, (uint64_t)s, dim_extra(bounce, 0));
        } else if (bounce < 3) {
            const float* v = sa.dims + s * sa.ndims + 10 * bounce;
            *lnum = v[0];
            *u0 = v[1];
            *u1 = v[2];
            *comp = v[3];
        } else {
            const float* v = sa.rng + sa.rng_base + 7 * s;
            *lnum = v[0];
            *u0 = v[1];
            *u1 = v[2];
            *comp = v[3];
        }
    }
    // the path's BSDF sample (uDir) and Russian roulette value
    __device__ void path_bsdf(float* u0, float* u1) const {
        if (!rc.stream) {
            *u0 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, kDimBsdf));
            *u1 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, kDimBsdf + 1));
        } else if (bounce < 3) {
            const float* v = sa.dims + s * sa.ndims + 10 * bounce;
            *u0 = v[7];
            *u1 = v[8];
        } else {
            const float* v = sa.rng + sa.rng_base + 7 * sa.count + (int64_t)sa.hit_rank[j] * (bounce > 3 ? 4 : 3);
            *u0 = v[0];
            *u1 = v[1];
        }
    }
    __device__ float path_rr() const {
        if (!rc.stream) return rnd(rc.seed, (uint64_t)s, dim_of(bounce, kDimRR));
        return sa.rng[sa.rng_base + 7 * sa.count + (int64_t)sa.hit_rank[j] * 4 + 3];
    }
};

// One queue entry: shade the hit, fill its shadow slots, its bounce slot and
// its emission (camera hits on emitting triangles).  A gather-bound kernel:
// 8 CTAs per SM (64 registers) measured best of 4, 5, 6 and 8 on the path
// frame (1,173 / 1,189 / 1,198 / 1,202 Mrays/s).
__global__ void __launch_bounds__(128, 8)
    shade_kernel(RenderConst rc, StreamArgs sa, int bounce, int64_t nq, const int32_t* __restrict__ qidx,
                             const float4* __restrict__ qo, const float4* __restrict__ qd,
                             const int32_t* __restrict__ prim, const float* __restrict__ th,
                             const float* __restrict__ b1v, const float* __restrict__ b2v,
                             const float* __restrict__ tri9, const float* __restrict__ uv6,
                             float* __restrict__ beta, int kslots, float4* __restrict__ so,
                             float4* __restrict__ sd, float* __restrict__ scontrib,
                             uint8_t* __restrict__ sflag, float4* __restrict__ no,
                             float4* __restrict__ nd_, uint8_t* __restrict__ nflag, float* __restrict__ emit,
                             int* __restrict__ rstat) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    for (int k = 0; k < kslots; ++k) sflag[j * kslots + k] = 0;
    nflag[j] = 0;
    emit[3 * j] = emit[3 * j + 1] = emit[3 * j + 2] = 0.f;
    const int32_t pr = prim[j];
    if (pr < 0) return;  // miss: no environment light
    const int64_t s = qidx[j];
    const Draws dr{rc, sa, s, j, bounce};
    const float4 o4 = qo[j], d4 = qd[j];
    const V3 ro = v3(o4.x, o4.y, o4.z), rdir = v3(d4.x, d4.y, d4.z);
    const float t = th[j];
    const HitDG g = hit_dg(tri9 + 9 * (int64_t)pr, uv6 ? uv6 + 6 * (int64_t)pr : nullptr, ro, rdir, t,
                           b1v[j], b2v[j]);
    const float eps = __fmul_rn(1e-3f, t);  // rayEpsilon (shapes/trianglemesh.cpp:190)
    Frame fr;
    fr.nn = g.nn;
    fr.sn = vnormalize(g.dpdu);
    fr.tn = vcross(fr.nn, fr.sn);
    const V3 ng = g.nn;
    const V3 wo = vneg(rdir);
    // Intersection::Le at camera hits (DiffuseAreaLight::L, lights/diffuse.h:43-45)
    if (bounce == 0) {
        for (int l = 0; l < rc.nlights; ++l) {
            const DevLight& lt = rc.lights[l];
            if (lt.type == PBG_LIGHT_MESH && pr >= lt.first && pr < lt.first + lt.ntri && vdot(g.nn, wo) > 0.f) {
                emit[3 * j] = lt.L[0];
                emit[3 * j + 1] = lt.L[1];
                emit[3 * j + 2] = lt.L[2];
            }
        }
    }
    const V3 R = v3(rc.albedo[0], rc.albedo[1], rc.albedo[2]);
    const V3 fR = v3(__fmul_rn(R.x, kInvPi), __fmul_rn(R.y, kInvPi), __fmul_rn(R.z, kInvPi));
    const V3 bt = v3(beta[3 * s], beta[3 * s + 1], beta[3 * s + 2]);
    const float won = vdot(wo, ng);
    const V3 wol = fr.to_local(wo);

    // Direct lighting: every light and sample (directlighting) or one light
    // sample (path).
    const bool all = rc.integrator == PBG_INTEGRATOR_DIRECT;
    int slot = 0;
    int first_light = 0, last_light = rc.nlights;
    float pu0 = 0.f, pu1 = 0.f, pcomp = 0.f;
    if (!all && rc.nlights > 0) {
        // UniformSampleOneLight: lightNum = min(Floor2Int(u * nLights), nLights - 1)
        float lnum;
        dr.path_light(&lnum, &pu0, &pu1, &pcomp);
        first_light = min((int)floorf(__fmul_rn(lnum, (float)rc.nlights)), rc.nlights - 1);
        last_light = first_light + 1;
    }
    for (int l = first_light; l < last_light; ++l) {
        const DevLight& lt = rc.lights[l];
        const int ns = all ? (lt.type == PBG_LIGHT_POINT ? 1 : max(lt.nsamples, 1)) : 1;
        for (int q = 0; q < ns; ++q, ++slot) {
            float u1, u2, comp;
            if (all) {
                dr.direct_light(slot, q, &u1, &u2, &comp);
            } else {
                u1 = pu0;
                u2 = pu1;
                comp = pcomp;
            }
            V3 wi, Li;
            float pdf;
            float4 o_, d_;
            if (slot >= kslots) break;
            if (!sample_light(rc, lt, tri9, uv6, g.p, eps, u1, u2, comp, &wi, &Li, &pdf, &o_, &d_)) continue;
            if (!(pdf > 0.f) || (Li.x == 0.f && Li.y == 0.f && Li.z == 0.f)) continue;
            const bool refl = __fmul_rn(vdot(wi, ng), won) > 0.f;
            if (!refl) continue;  // f = 0: Lambertian reflects only
            const float absdot = fabsf(vdot(wi, fr.nn));
            const V3 fL = v3(__fmul_rn(fR.x, Li.x), __fmul_rn(fR.y, Li.y), __fmul_rn(fR.z, Li.z));
            V3 c;
            if (lt.type == PBG_LIGHT_POINT) {
                if (all) {  // f * Li * AbsDot / lightPdf
                    c = v3(__fdiv_rn(__fmul_rn(fL.x, absdot), pdf), __fdiv_rn(__fmul_rn(fL.y, absdot), pdf),
                           __fdiv_rn(__fmul_rn(fL.z, absdot), pdf));
                } else {    // f * Li * (AbsDot / lightPdf)
                    const float w = __fdiv_rn(absdot, pdf);
                    c = v3(__fmul_rn(fL.x, w), __fmul_rn(fL.y, w), __fmul_rn(fL.z, w));
                }
            } else {
                const V3 wil = fr.to_local(wi);
                const bool same = __fmul_rn(wol.z, wil.z) > 0.f;
                const float bpdf = same ? __fmul_rn(fabsf(wil.z), kInvPi) : 0.f;
                // PowerHeuristic(1, pdf, 1, bpdf)
                const float f2 = __fmul_rn(pdf, pdf), g2 = __fmul_rn(bpdf, bpdf);
                const float weight = __fdiv_rn(f2, __fadd_rn(f2, g2));
                if (all) {  // f * Li * AbsDot * weight / lightPdf
                    c = v3(__fdiv_rn(__fmul_rn(__fmul_rn(fL.x, absdot), weight), pdf),
                           __fdiv_rn(__fmul_rn(__fmul_rn(fL.y, absdot), weight), pdf),
                           __fdiv_rn(__fmul_rn(__fmul_rn(fL.z, absdot), weight), pdf));
                } else {    // f * Li * (AbsDot * weight / lightPdf)
                    const float w = __fdiv_rn(__fmul_rn(absdot, weight), pdf);
                    c = v3(__fmul_rn(fL.x, w), __fmul_rn(fL.y, w), __fmul_rn(fL.z, w));
                }
            }
            if (!all) {  // Ld *= nLights, then L += pathThroughput * Ld
                const float fl = (float)rc.nlights;
                c = v3(__fmul_rn(c.x, fl), __fmul_rn(c.y, fl), __fmul_rn(c.z, fl));
                c = v3(__fmul_rn(bt.x, c.x), __fmul_rn(bt.y, c.y), __fmul_rn(bt.z, c.z));
            }
            const int64_t si = j * kslots + slot;
            so[si] = o_;
            sd[si] = d_;
            scontrib[3 * si] = c.x;
            scontrib[3 * si + 1] = c.y;
            scontrib[3 * si + 2] = c.z;
            sflag[si] = 1;
        }
    }
    if (rc.integrator != PBG_INTEGRATOR_PATH) return;

    // BSDF sample for the next vertex (Lambertian::Sample_f, cosine-weighted
    // through ConcentricSampleDisk, core/montecarlo.cpp).
    float u1, u2;
    dr.path_bsdf(&u1, &u2);
    float sx = __fsub_rn(__fmul_rn(2.f, u1), 1.f), sy = __fsub_rn(__fmul_rn(2.f, u2), 1.f);
    float dx = 0.f, dy = 0.f;
    if (!(sx == 0.f && sy == 0.f)) {
        float r, theta;
        if (sx >= -sy) {
            if (sx > sy) {
                r = sx;
                theta = sy > 0.f ? __fdiv_rn(sy, r) : __fadd_rn(8.f, __fdiv_rn(sy, r));
            } else {
                r = sy;
                theta = __fsub_rn(2.f, __fdiv_rn(sx, r));
            }
        } else {
            if (sx <= sy) {
                r = -sx;
                theta = __fsub_rn(4.f, __fdiv_rn(sy, r));
            } else {
                r = -sy;
                theta = __fadd_rn(6.f, __fdiv_rn(sx, r));
            }
        }
        float st, ct;
        if (rc.stream) {
            // theta *= M_PI / 4.f is a double product rounded to float; the
            // reference's cosf/sinf come from the host's libm, here the
            // correctly rounded value (one double evaluation, rounded once)
            theta = __double2float_rn(__dmul_rn((double)theta, 0.78539816339744830962));
            double ds, dc;
            sincos((double)theta, &ds, &dc);
            st = __double2float_rn(ds);
            ct = __double2float_rn(dc);
        } else {
            theta = __fmul_rn(theta, 0.785398163397448309616f);
            own_sincos(theta, &st, &ct);
        }
        dx = __fmul_rn(r, ct);
        dy = __fmul_rn(r, st);
    }
    V3 wil = v3(dx, dy, __fsqrt_rn(fmaxf(0.f, __fsub_rn(__fsub_rn(1.f, __fmul_rn(dx, dx)), __fmul_rn(dy, dy)))));
    if (wol.z < 0.f) wil.z = -wil.z;
    const bool same = __fmul_rn(wol.z, wil.z) > 0.f;
    const float pdf = same ? __fmul_rn(fabsf(wil.z), kInvPi) : 0.f;
    const V3 wi = fr.to_world(wil);
    const bool refl = __fmul_rn(vdot(wi, ng), won) > 0.f;
    if (!refl || !(pdf > 0.f)) {
        // the reference keeps such a ray alive with its old direction
        // (integrators/path.cpp:112-113); a stream render stops matching it
        if (rc.stream) atomicAdd(&rstat[0], 1);
        return;
    }
    const float absdot = fabsf(vdot(wi, fr.nn));
    // pathThroughput *= f * AbsDot(wi, n) / pdf
    V3 nb = v3(__fmul_rn(bt.x, __fdiv_rn(__fmul_rn(fR.x, absdot), pdf)),
               __fmul_rn(bt.y, __fdiv_rn(__fmul_rn(fR.y, absdot), pdf)),
               __fmul_rn(bt.z, __fdiv_rn(__fmul_rn(fR.z, absdot), pdf)));
    if (bounce > 3) {  // Russian roulette (integrators/path.cpp:117-124)
        const float y = __fadd_rn(__fadd_rn(__fmul_rn(0.212671f, nb.x), __fmul_rn(0.715160f, nb.y)),
                                  __fmul_rn(0.072169f, nb.z));
        const float cont = fminf(0.5f, y);
        if (dr.path_rr() > cont) return;
        nb = v3(__fdiv_rn(nb.x, cont), __fdiv_rn(nb.y, cont), __fdiv_rn(nb.z, cont));
    }
    if (bounce == rc.max_depth) return;
    beta[3 * s] = nb.x;
    beta[3 * s + 1] = nb.y;
    beta[3 * s + 2] = nb.z;
    no[j] = make_float4(g.p.x, g.p.y, g.p.z, eps);
    nd_[j] = make_float4(wi.x, wi.y, wi.z, INFINITY);
    nflag[j] = 1;
}

// Triangle-emitter tables: Triangle::Area (shapes/trianglemesh.cpp:276-282)
// in ShapeSet order, the total area and the Distribution1D CDF
// (core/montecarlo.h:48-70), in pbrt's float arithmetic.  One thread.
__global__ void emitter_setup_kernel(const float* __restrict__ tri9, int first, int n, float* __restrict__ tab) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float sum = 0.f;
    for (int i = 0; i < n; ++i) {
        const float* v = tri9 + 9 * shape_tri(first, n, i);
        const V3 p1 = tri_vertex(v, 0);
        const V3 c = vcross(vsub(tri_vertex(v, 1), p1), vsub(tri_vertex(v, 2), p1));
        const float a = __fmul_rn(0.5f, vlen(c));
        tab[i] = a;
        sum = __fadd_rn(sum, a);
    }
    float* cdf = tab + n;
    cdf[0] = 0.f;
    for (int i = 1; i <= n; ++i) cdf[i] = __fadd_rn(cdf[i - 1], __fdiv_rn(tab[i - 1], (float)n));
    const float integral = cdf[n];
    for (int i = 1; i <= n; ++i)
        cdf[i] = integral == 0.f ? __fdiv_rn((float)i, (float)n) : __fdiv_rn(cdf[i], integral);
    cdf[n + 1] = sum;
}

// Order-preserving compaction, phase 1: per-block count of set flags.
__global__ void flag_count_kernel(const uint8_t* __restrict__ flag, int64_t n, uint32_t* __restrict__ counts) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = __syncthreads_count(i < n && flag[i] != 0);
    if (threadIdx.x == 0) counts[blockIdx.x] = (uint32_t)c;
}

// Phase 2 (after a scan of the block counts): rank inside the block from
// warp ballots, then gather.  pos[i] receives the dense index or -1.
template <typename Fn>
__device__ __forceinline__ void compact_rank(const uint8_t* flag, int64_t n, const uint32_t* offs,
                                             int32_t* pos, Fn&& emit) {
    __shared__ uint32_t warp_base[32];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool f = i < n && flag[i] != 0;
    const unsigned b = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_base[warp] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            const uint32_t c = warp_base[w];
            warp_base[w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (i >= n) return;
    if (!f) {
        if (pos) pos[i] = -1;
        return;
    }
    const uint32_t dst = offs[blockIdx.x] + warp_base[warp] + __popc(b & ((1u << lane) - 1u));
    if (pos) pos[i] = (int32_t)dst;
    emit(i, dst);
}

__global__ void compact_shadow_kernel(const uint8_t* __restrict__ flag, int64_t n,
                                      const uint32_t* __restrict__ offs, const float4* __restrict__ so,
                                      const float4* __restrict__ sd, float4* __restrict__ qo,
                                      float4* __restrict__ qd, int32_t* __restrict__ pos) {
    compact_rank(flag, n, offs, pos, [&](int64_t i, uint32_t dst) {
        qo[dst] = so[i];
        qd[dst] = sd[i];
    });
}

__global__ void compact_bounce_kernel(const uint8_t* __restrict__ flag, int64_t n,
                                      const uint32_t* __restrict__ offs, const int32_t* __restrict__ qidx,
                                      const float4* __restrict__ no, const float4* __restrict__ nd_,
                                      int32_t* __restrict__ qidx_out, float4* __restrict__ qo,
                                      float4* __restrict__ qd) {
    compact_rank(flag, n, offs, nullptr, [&](int64_t i, uint32_t dst) {
        qidx_out[dst] = qidx[i];
        qo[dst] = no[i];
        qd[dst] = nd_[i];
    });
}

// Stream renders, path bounces >= 3: each queue entry's rank among the
// entries that hit (the order in which the reference's BSDF loop draws).
__global__ void hit_flag_kernel(const int32_t* __restrict__ prim, int64_t n, uint8_t* __restrict__ flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = prim[i] >= 0 ? 1 : 0;
}

__global__ void hit_rank_kernel(const uint8_t* __restrict__ flag, int64_t n, const uint32_t* __restrict__ offs,
                                int32_t* __restrict__ rank) {
    compact_rank(flag, n, offs, rank, [](int64_t, uint32_t) {});
}

// Unoccluded shadow contributions and emission, added per entry in slot
// order.  directlighting: Ld = the sum over every light and sample
// (UniformSampleAllLights' batch form, core/integrator.cpp:73-122, does not
// divide by the sample count), L += Ld, then L += Le
// (integrators/directlighting.cpp:112-133); path: L += Le at the camera
// vertex, then the single slot, which already carries beta * nLights * Ld.
__global__ void resolve_kernel(RenderConst rc, int64_t nq, int kslots, const int32_t* __restrict__ qidx,
                               const uint8_t* __restrict__ sflag, const int32_t* __restrict__ spos,
                               const uint8_t* __restrict__ occ, const float* __restrict__ scontrib,
                               const float* __restrict__ emit, float* __restrict__ L) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    const int64_t s = qidx[j];
    float lx = L[3 * s], ly = L[3 * s + 1], lz = L[3 * s + 2];
    const float ex = emit[3 * j], ey = emit[3 * j + 1], ez = emit[3 * j + 2];
    if (rc.integrator == PBG_INTEGRATOR_DIRECT) {
        float ax = 0.f, ay = 0.f, az = 0.f;
        for (int k = 0; k < kslots; ++k) {
            const int64_t si = j * kslots + k;
            if (!sflag[si] || occ[spos[si]]) continue;
            ax = __fadd_rn(ax, scontrib[3 * si]);
            ay = __fadd_rn(ay, scontrib[3 * si + 1]);
            az = __fadd_rn(az, scontrib[3 * si + 2]);
        }
        lx = __fadd_rn(__fadd_rn(lx, ax), ex);
        ly = __fadd_rn(__fadd_rn(ly, ay), ey);
        lz = __fadd_rn(__fadd_rn(lz, az), ez);
    } else {
        lx = __fadd_rn(lx, ex);
        ly = __fadd_rn(ly, ey);
        lz = __fadd_rn(lz, ez);
        for (int k = 0; k < kslots; ++k) {
            const int64_t si = j * kslots + k;
            if (!sflag[si] || occ[spos[si]]) continue;
            lx = __fadd_rn(lx, scontrib[3 * si]);
            ly = __fadd_rn(ly, scontrib[3 * si + 1]);
            lz = __fadd_rn(lz, scontrib[3 * si + 2]);
        }
    }
    L[3 * s] = lx;
    L[3 * s + 1] = ly;
    L[3 * s + 2] = lz;
}

// ImageFilm: RGB -> XYZ per sample, summed in sample order, back to RGB,
// divided by the weight sum, clamped at zero (film/image.cpp).  A sample
// whose radiance breadthFirst::Li rejects (NaN, luminance below -1e-5 or
// infinite, renderers/breadth-first.cpp:196-213) adds black.  Samples of
// pixel p: [off[p], off[p + 1]) of idx when a list is given (stream
// renders), else the spp consecutive samples p * spp ...
__device__ __forceinline__ void film_add(const float* L, int64_t s, float* X, float* Y, float* Z, float* w) {
    float r = L[3 * s], g = L[3 * s + 1], b = L[3 * s + 2];
    const float lum = __fadd_rn(__fadd_rn(__fmul_rn(0.212671f, r), __fmul_rn(0.715160f, g)), __fmul_rn(0.072169f, b));
    if (isnan(r) || isnan(g) || isnan(b) || lum < -1e-5f || isinf(lum)) r = g = b = 0.f;
    const float x = __fadd_rn(__fadd_rn(__fmul_rn(0.412453f, r), __fmul_rn(0.357580f, g)), __fmul_rn(0.180423f, b));
    const float y = __fadd_rn(__fadd_rn(__fmul_rn(0.212671f, r), __fmul_rn(0.715160f, g)), __fmul_rn(0.072169f, b));
    const float z = __fadd_rn(__fadd_rn(__fmul_rn(0.019334f, r), __fmul_rn(0.119193f, g)), __fmul_rn(0.950227f, b));
    *X = __fadd_rn(*X, x);
    *Y = __fadd_rn(*Y, y);
    *Z = __fadd_rn(*Z, z);
    *w = __fadd_rn(*w, 1.f);
}

__global__ void film_kernel(int64_t npix, int spp, const int32_t* __restrict__ off, const int32_t* __restrict__ idx,
                            const float* __restrict__ L, float* __restrict__ rgb) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float X = 0.f, Y = 0.f, Z = 0.f, w = 0.f;
    if (off) {
        for (int32_t k = off[p]; k < off[p + 1]; ++k) film_add(L, idx[k], &X, &Y, &Z, &w);
    } else {
        for (int k = 0; k < spp; ++k) film_add(L, p * spp + k, &X, &Y, &Z, &w);
    }
    float R = __fsub_rn(__fsub_rn(__fmul_rn(3.240479f, X), __fmul_rn(1.537150f, Y)), __fmul_rn(0.498535f, Z));
    float G = __fadd_rn(__fadd_rn(__fmul_rn(-0.969256f, X), __fmul_rn(1.875991f, Y)), __fmul_rn(0.041556f, Z));
    float B = __fadd_rn(__fsub_rn(__fmul_rn(0.055648f, X), __fmul_rn(0.204043f, Y)), __fmul_rn(1.057311f, Z));
    if (w != 0.f) {
        const float inv = __frcp_rn(w);
        R = fmaxf(0.f, __fmul_rn(R, inv));
        G = fmaxf(0.f, __fmul_rn(G, inv));
        B = fmaxf(0.f, __fmul_rn(B, inv));
    }
    rgb[3 * p] = R;
    rgb[3 * p + 1] = G;
    rgb[3 * p + 2] = B;
}

// ------------------------------------------------------------------ host

int scan_counts(pbg_scene* s, uint32_t* a, int64_t m, cudaStream_t st);

// One bounce's shadow queue: its slots (shade), the compacted rays, their
// occlusion and the bounce's emission (resolve).  Path frames on ray-bvh
// and naive scenes keep two, so that a bounce's shadow traversal and resolve
// run on a second stream beside the next bounce's nearest-hit traversal.
struct ShadowSet {
    DeviceBuffer so, sd, scontrib, sflag, spos, sqo, sqd, occ, emit;
    void release_all() {
        DeviceBuffer* all[] = {&so, &sd, &scontrib, &sflag, &spos, &sqo, &sqd, &occ, &emit};
        for (DeviceBuffer* b : all) release(*b);
    }
};

struct RenderBuffers {
    DeviceBuffer o4, d4, qidx, L, beta, prim, t, b1, b2, no, nd, nflag, qidx2, o42, d42, counts, rgb, rstat,
        ltab, simg, sdims, srng, hflag, hrank, foff, fidx;
    ShadowSet sh[2];
    cudaStream_t side = nullptr;           // the shadow stream of overlapped frames
    cudaEvent_t ready[2] = {}, resolved[2] = {};
    ~RenderBuffers() {
        DeviceBuffer* all[] = {&o4,    &d4,     &qidx,  &L,     &beta, &prim,  &t,     &b1,   &b2,
                               &no,    &nd,     &nflag, &qidx2, &o42,  &d42,   &counts, &rgb, &rstat,
                               &ltab,  &simg,   &sdims, &srng,  &hflag, &hrank, &foff,  &fidx};
        for (DeviceBuffer* b : all) release(*b);
        for (ShadowSet& x : sh) x.release_all();
        for (int k = 0; k < 2; ++k) {
            if (ready[k]) cudaEventDestroy(ready[k]);
            if (resolved[k]) cudaEventDestroy(resolved[k]);
        }
        if (side) cudaStreamDestroy(side);
    }
};

void render_free(pbg_scene* s) {
    delete s->render_bufs;
    s->render_bufs = nullptr;
}

static int compact_count(pbg_scene* s, const uint8_t* flag, int64_t n, uint32_t* counts, int64_t* total,
                         cudaStream_t st) {
    const int64_t blocks = (n + 255) / 256;
    flag_count_kernel<<<(unsigned)blocks, 256, 0, st>>>(flag, n, counts);
    PBG_CUDA(cudaGetLastError());
    uint32_t last_count = 0;
    PBG_CUDA(cudaMemcpyAsync(&last_count, counts + blocks - 1, 4, cudaMemcpyDeviceToHost, st));
    int rc = scan_counts(s, counts, blocks, st);
    if (rc) return rc;
    uint32_t last_off = 0;
    PBG_CUDA(cudaMemcpyAsync(&last_off, counts + blocks - 1, 4, cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    *total = (int64_t)last_off + last_count;
    s->counters.kernel_launches += 1;
    return PBG_OK;
}

// The pixels a sample at (x, y) adds to: ImageFilm::AddSample's footprint of
// the box filter of radius 0.5 (film/image.cpp), clipped to the image.
static void film_footprint(float x, float y, int xres, int yres, int* x0, int* x1, int* y0, int* y1) {
    const float dx = x - 0.5f, dy = y - 0.5f;
    *x0 = std::max((int)std::ceil(dx - 0.5f), 0);
    *x1 = std::min((int)std::floor(dx + 0.5f), xres - 1);
    *y0 = std::max((int)std::ceil(dy - 0.5f), 0);
    *y1 = std::min((int)std::floor(dy + 0.5f), yres - 1);
}

int render(pbg_scene* s, const pbg_camera* cam, const pbg_light* lights, int32_t nlights,
           const pbg_render_params* prm, const pbg_sample_stream* stream, float* rgb_host,
           pbg_render_stats* stats) {
    if (!cam || !prm || nlights < 0 || nlights > 4 || (nlights > 0 && !lights) || !rgb_host ||
        cam->xres <= 0 || cam->yres <= 0 || prm->spp_x <= 0 || prm->spp_y <= 0 ||
        (prm->integrator != PBG_INTEGRATOR_DIRECT && prm->integrator != PBG_INTEGRATOR_PATH)) {
        set_last_error("pbg_render: bad arguments");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    RenderConst rc{};
    memcpy(rc.r2c, cam->raster_to_camera, sizeof(rc.r2c));
    memcpy(rc.c2w, cam->camera_to_world, sizeof(rc.c2w));
    rc.xres = cam->xres;
    rc.yres = cam->yres;
    rc.spp_x = prm->spp_x;
    rc.spp_y = prm->spp_y;
    rc.spp = prm->spp_x * prm->spp_y;
    rc.jitter = prm->jitter;
    rc.max_depth = prm->max_depth > 0 ? prm->max_depth : 5;
    rc.integrator = prm->integrator;
    rc.seed = prm->seed;
    rc.stream = stream != nullptr;
    for (int k = 0; k < 3; ++k) rc.albedo[k] = prm->albedo[k];
    rc.nlights = nlights;
    int kslots = 0, ltab_floats = 0;
    for (int l = 0; l < nlights; ++l) {
        const pbg_light& in = lights[l];
        DevLight& d = rc.lights[l];
        d.type = in.type;
        d.nsamples = in.nsamples > 0 ? in.nsamples : 1;
        for (int k = 0; k < 3; ++k) {
            d.pos[k] = in.pos[k];
            d.I[k] = in.intensity[k];
            d.q0[k] = in.quad[k];
            d.e1[k] = in.quad[3 + k] - in.quad[k];
            d.e3[k] = in.quad[9 + k] - in.quad[k];
            d.L[k] = in.radiance[k];
        }
        if (in.type == PBG_LIGHT_MESH) {
            if (in.ntri <= 0 || in.ntri > 64 || in.first_tri < 0 || (int64_t)in.first_tri + in.ntri > s->ntri) {
                set_last_error("pbg_render: a triangle emitter needs 1..64 triangles of the scene");
                return PBG_ERR_INVALID_ARGUMENT;
            }
            d.first = in.first_tri;
            d.ntri = in.ntri;
            d.tab = ltab_floats;
            ltab_floats += 2 * in.ntri + 2;
        } else if (in.type != PBG_LIGHT_POINT && in.type != PBG_LIGHT_QUAD) {
            set_last_error("pbg_render: unknown light type");
            return PBG_ERR_INVALID_ARGUMENT;
        }
        const double cx = (double)d.e1[1] * d.e3[2] - (double)d.e1[2] * d.e3[1];
        const double cy = (double)d.e1[2] * d.e3[0] - (double)d.e1[0] * d.e3[2];
        const double cz = (double)d.e1[0] * d.e3[1] - (double)d.e1[1] * d.e3[0];
        const double len = std::sqrt(cx * cx + cy * cy + cz * cz);
        d.area = (float)len;
        d.n[0] = len > 0 ? (float)(cx / len) : 0.f;
        d.n[1] = len > 0 ? (float)(cy / len) : 0.f;
        d.n[2] = len > 0 ? (float)(cz / len) : 0.f;
        if (prm->integrator == PBG_INTEGRATOR_DIRECT)
            kslots += d.type == PBG_LIGHT_POINT ? 1 : d.nsamples;
        else if (l == 0)
            kslots = 1;
    }
    if (kslots == 0) kslots = 1;
    const int64_t npix = (int64_t)cam->xres * cam->yres;
    const int64_t n = stream ? stream->count : npix * rc.spp;
    if (n <= 0 || n > (int64_t)INT32_MAX / std::max(kslots, 1)) {
        set_last_error("pbg_render: image too large for one batch, or an empty sample stream");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    if (stream) {
        const int need = prm->integrator == PBG_INTEGRATOR_PATH ? 30 : 6 * kslots;
        if (!stream->image_xy || !stream->dims || stream->ndims < need || stream->nrng < 0 ||
            (stream->nrng > 0 && !stream->rng)) {
            set_last_error("pbg_render_stream: the stream needs image positions, the sample values of its layout "
                           "(30 per sample for path, 6 per light sample for directlighting) and its RNG draws");
            return PBG_ERR_INVALID_ARGUMENT;
        }
    }
    cudaStream_t st = s->stream;
    if (!s->render_bufs) s->render_bufs = new RenderBuffers();
    RenderBuffers& B = *s->render_bufs;  // grown on demand, kept for the next frame
    int r;
    const size_t nk = (size_t)n * kslots;
    // Overlapped bounces (path frames on ray-bvh and naive scenes): each
    // bounce's shadow traversal and resolve go to a second stream, beside
    // the next bounce's nearest-hit traversal and shading.  rayhierarchy
    // batches share the scene's status words, and a learned ordering that
    // serves nearest-hit batches shares its prediction and record buffers
    // with the any-hit ones, so those frames stay serial.
    const bool overlap = prm->integrator == PBG_INTEGRATOR_PATH &&
                         (s->accel == PBG_ACCEL_RAYBVH || s->accel == PBG_ACCEL_NAIVE) &&
                         !(s->learn && s->learn->enabled && (s->learn->queries & 1));
    if ((r = ensure(B.o4, n * 16)) || (r = ensure(B.d4, n * 16)) || (r = ensure(B.qidx, n * 4)) ||
        (r = ensure(B.L, n * 12)) || (r = ensure(B.beta, n * 12)) || (r = ensure(B.prim, n * 4)) ||
        (r = ensure(B.t, n * 4)) || (r = ensure(B.b1, n * 4)) || (r = ensure(B.b2, n * 4)) ||
        (r = ensure(B.no, n * 16)) || (r = ensure(B.nd, n * 16)) || (r = ensure(B.nflag, n)) ||
        (r = ensure(B.qidx2, n * 4)) || (r = ensure(B.o42, n * 16)) || (r = ensure(B.d42, n * 16)) ||
        (r = ensure(B.counts, ((nk + 255) / 256 + 64) * 4 + 4096)) || (r = ensure(B.rgb, npix * 12)) ||
        (r = ensure(B.rstat, 16)) || (r = ensure(B.ltab, (size_t)std::max(ltab_floats, 1) * 4)))
        return r;
    for (int k = 0; k < (overlap ? 2 : 1); ++k) {
        ShadowSet& X = B.sh[k];
        if ((r = ensure(X.so, nk * 16)) || (r = ensure(X.sd, nk * 16)) || (r = ensure(X.scontrib, nk * 12)) ||
            (r = ensure(X.sflag, nk)) || (r = ensure(X.spos, nk * 4)) || (r = ensure(X.sqo, nk * 16)) ||
            (r = ensure(X.sqd, nk * 16)) || (r = ensure(X.occ, nk)) || (r = ensure(X.emit, n * 12)))
            return r;
    }
    // a frame that ended early on an error may have left work on the side stream
    if (B.side) PBG_CUDA(cudaStreamSynchronize(B.side));
    if (overlap && !B.side) {
        PBG_CUDA(cudaStreamCreateWithFlags(&B.side, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            PBG_CUDA(cudaEventCreateWithFlags(&B.ready[k], cudaEventDisableTiming));
            PBG_CUDA(cudaEventCreateWithFlags(&B.resolved[k], cudaEventDisableTiming));
        }
    }
    PBG_CUDA(cudaMemsetAsync(B.rstat.ptr, 0, 16, st));
    rc.ltab = (const float*)B.ltab.ptr;
    for (int l = 0; l < nlights; ++l)
        if (rc.lights[l].type == PBG_LIGHT_MESH) {
            emitter_setup_kernel<<<1, 32, 0, st>>>((const float*)s->tri9.ptr, rc.lights[l].first, rc.lights[l].ntri,
                                                   (float*)B.ltab.ptr + rc.lights[l].tab);
            PBG_CUDA(cudaGetLastError());
            s->counters.kernel_launches += 1;
        }
    StreamArgs sa{};
    const int32_t* film_off = nullptr;
    const int32_t* film_idx = nullptr;
    if (stream) {
        // the caller's sample values, and each pixel's samples in order
        const size_t nd = (size_t)stream->ndims;
        std::vector<int32_t> cnt(npix + 1, 0);
        for (int64_t i = 0; i < n; ++i) {
            int x0, x1, y0, y1;
            film_footprint(stream->image_xy[2 * i], stream->image_xy[2 * i + 1], cam->xres, cam->yres, &x0, &x1, &y0, &y1);
            for (int y = y0; y <= y1; ++y)
                for (int x = x0; x <= x1; ++x) cnt[(int64_t)y * cam->xres + x + 1]++;
        }
        for (int64_t p = 0; p < npix; ++p) cnt[p + 1] += cnt[p];
        std::vector<int32_t> idx(std::max<int32_t>(cnt[npix], 1)), fill(cnt.begin(), cnt.end() - 1);
        for (int64_t i = 0; i < n; ++i) {
            int x0, x1, y0, y1;
            film_footprint(stream->image_xy[2 * i], stream->image_xy[2 * i + 1], cam->xres, cam->yres, &x0, &x1, &y0, &y1);
            for (int y = y0; y <= y1; ++y)
                for (int x = x0; x <= x1; ++x) idx[fill[(int64_t)y * cam->xres + x]++] = (int32_t)i;
        }
        if ((r = ensure(B.simg, n * 8)) || (r = ensure(B.sdims, n * nd * 4)) ||
            (r = ensure(B.srng, (size_t)std::max<int64_t>(stream->nrng, 1) * 4)) || (r = ensure(B.hflag, n)) ||
            (r = ensure(B.hrank, n * 4)) || (r = ensure(B.foff, (npix + 1) * 4)) ||
            (r = ensure(B.fidx, idx.size() * 4)))
            return r;
        PBG_CUDA(cudaMemcpyAsync(B.simg.ptr, stream->image_xy, n * 8, cudaMemcpyHostToDevice, st));
        PBG_CUDA(cudaMemcpyAsync(B.sdims.ptr, stream->dims, n * nd * 4, cudaMemcpyHostToDevice, st));
        if (stream->nrng > 0)
            PBG_CUDA(cudaMemcpyAsync(B.srng.ptr, stream->rng, stream->nrng * 4, cudaMemcpyHostToDevice, st));
        PBG_CUDA(cudaMemcpyAsync(B.foff.ptr, cnt.data(), (npix + 1) * 4, cudaMemcpyHostToDevice, st));
        PBG_CUDA(cudaMemcpyAsync(B.fidx.ptr, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, st));
        PBG_CUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
        sa.img = (const float*)B.simg.ptr;
        sa.dims = (const float*)B.sdims.ptr;
        sa.rng = (const float*)B.srng.ptr;
        sa.count = n;
        sa.nrng = stream->nrng;
        sa.ndims = stream->ndims;
        film_off = (const int32_t*)B.foff.ptr;
        film_idx = (const int32_t*)B.fidx.ptr;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    raygen_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        rc, sa, n, (float4*)B.o4.ptr, (float4*)B.d4.ptr, (int32_t*)B.qidx.ptr, (float*)B.L.ptr,
        (float*)B.beta.ptr);
    PBG_CUDA(cudaGetLastError());
    s->counters.kernel_launches += 1;
    pbg_render_stats stt{};
    stt.camera_rays = (uint64_t)n;
    int64_t nq = n;
    int64_t rng_base = 0;
    // queue arrays alternate between (qidx, o4, d4) and (qidx2, o42, d42)
    int32_t* qi = (int32_t*)B.qidx.ptr;
    float4* qo = (float4*)B.o4.ptr;
    float4* qd = (float4*)B.d4.ptr;
    int32_t* qi2 = (int32_t*)B.qidx2.ptr;
    float4* qo2 = (float4*)B.o42.ptr;
    float4* qd2 = (float4*)B.d42.ptr;
    // camera rays and their shadow rays are coherent, later bounces are not
    struct HintGuard {
        pbg_scene* s;
        ~HintGuard() { s->walk_hint = -1; }
    } hint_guard{s};
    cudaStream_t side = overlap ? B.side : st;
    bool pending[2] = {false, false};  // a resolve on the side stream still reads set k
    for (int bounce = 0; nq > 0; ++bounce) {
        s->walk_hint = bounce > 0 ? 1 : 0;
        const int k = overlap ? (bounce & 1) : 0;
        ShadowSet& X = B.sh[k];
        if ((r = pbg_intersect_device(s, (const float*)qo, (const float*)qd, nullptr, nq,
                                      (int32_t*)B.prim.ptr, (float*)B.t.ptr, (float*)B.b1.ptr,
                                      (float*)B.b2.ptr, st)))
            return r;
        stt.nearest_rays += (uint64_t)nq;
        const bool draws = stream && rc.integrator == PBG_INTEGRATOR_PATH && bounce >= 3;
        int64_t nhits = 0;
        if (draws) {
            hit_flag_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>((const int32_t*)B.prim.ptr, nq,
                                                                           (uint8_t*)B.hflag.ptr);
            PBG_CUDA(cudaGetLastError());
            s->counters.kernel_launches += 1;
            if ((r = compact_count(s, (const uint8_t*)B.hflag.ptr, nq, (uint32_t*)B.counts.ptr, &nhits, st))) return r;
            hit_rank_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(
                (const uint8_t*)B.hflag.ptr, nq, (const uint32_t*)B.counts.ptr, (int32_t*)B.hrank.ptr);
            PBG_CUDA(cudaGetLastError());
            s->counters.kernel_launches += 1;
            if (rng_base + 7 * n + nhits * (bounce > 3 ? 4 : 3) > stream->nrng) {
                set_last_error("pbg_render_stream: the stream's RNG draws ran out");
                return PBG_ERR_INVALID_ARGUMENT;
            }
            sa.rng_base = rng_base;
            sa.hit_rank = (const int32_t*)B.hrank.ptr;
        }
        const int64_t nslots = nq * kslots;
        // set k was last read by the resolve of two bounces ago
        if (pending[k]) PBG_CUDA(cudaStreamWaitEvent(st, B.resolved[k], 0));
        pending[k] = false;
        shade_kernel<<<(unsigned)((nq + 127) / 128), 128, 0, st>>>(
            rc, sa, bounce, nq, qi, qo, qd, (const int32_t*)B.prim.ptr, (const float*)B.t.ptr,
            (const float*)B.b1.ptr, (const float*)B.b2.ptr, (const float*)s->tri9.ptr,
            (const float*)s->uv6.ptr, (float*)B.beta.ptr, kslots, (float4*)X.so.ptr, (float4*)X.sd.ptr,
            (float*)X.scontrib.ptr, (uint8_t*)X.sflag.ptr, (float4*)B.no.ptr, (float4*)B.nd.ptr,
            (uint8_t*)B.nflag.ptr, (float*)X.emit.ptr, (int*)B.rstat.ptr);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 1;
        if (draws) rng_base += 7 * n + nhits * (bounce > 3 ? 4 : 3);
        // shadow queue
        int64_t nsh = 0;
        if ((r = compact_count(s, (const uint8_t*)X.sflag.ptr, nslots, (uint32_t*)B.counts.ptr, &nsh, st)))
            return r;
        compact_shadow_kernel<<<(unsigned)((nslots + 255) / 256), 256, 0, st>>>(
            (const uint8_t*)X.sflag.ptr, nslots, (const uint32_t*)B.counts.ptr, (const float4*)X.so.ptr,
            (const float4*)X.sd.ptr, (float4*)X.sqo.ptr, (float4*)X.sqd.ptr, (int32_t*)X.spos.ptr);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 1;
        if (overlap) {  // the shadow rays and this bounce's resolve on the side stream
            PBG_CUDA(cudaEventRecord(B.ready[k], st));
            PBG_CUDA(cudaStreamWaitEvent(side, B.ready[k], 0));
        }
        if (nsh > 0) {
            if (overlap) std::swap(s->work, s->alt);  // its own walk counter, beside the nearest-hit walk
            r = pbg_occluded_device(s, (const float*)X.sqo.ptr, (const float*)X.sqd.ptr, nullptr, nsh,
                                    (uint8_t*)X.occ.ptr, side);
            if (overlap) std::swap(s->work, s->alt);
            if (r) return r;
        }
        stt.shadow_rays += (uint64_t)nsh;
        resolve_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, side>>>(
            rc, nq, kslots, qi, (const uint8_t*)X.sflag.ptr, (const int32_t*)X.spos.ptr,
            (const uint8_t*)X.occ.ptr, (const float*)X.scontrib.ptr, (const float*)X.emit.ptr, (float*)B.L.ptr);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 1;
        if (overlap) {
            PBG_CUDA(cudaEventRecord(B.resolved[k], side));
            pending[k] = true;
        }
        if (rc.integrator != PBG_INTEGRATOR_PATH) break;
        // bounce queue
        int64_t nn = 0;
        if ((r = compact_count(s, (const uint8_t*)B.nflag.ptr, nq, (uint32_t*)B.counts.ptr, &nn, st)))
            return r;
        // the resolve above reads this bounce's queue indices, which the
        // compaction after the next bounce overwrites: it waits there (below)
        if (overlap && pending[k ^ 1]) {
            PBG_CUDA(cudaStreamWaitEvent(st, B.resolved[k ^ 1], 0));
            pending[k ^ 1] = false;
        }
        compact_bounce_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(
            (const uint8_t*)B.nflag.ptr, nq, (const uint32_t*)B.counts.ptr, qi, (const float4*)B.no.ptr,
            (const float4*)B.nd.ptr, qi2, qo2, qd2);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 1;
        std::swap(qi, qi2);
        std::swap(qo, qo2);
        std::swap(qd, qd2);
        nq = nn;
        stt.bounces = (uint64_t)bounce + 1;
    }
    for (int k = 0; k < 2; ++k)  // the last resolves add to L before the film reads it
        if (pending[k]) PBG_CUDA(cudaStreamWaitEvent(st, B.resolved[k], 0));
    // online training of the learned ordering on this frame's records
    if (s->learn && s->learn->enabled && (r = learn_train(s, 0, st))) return r;
    film_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(npix, rc.spp, film_off, film_idx,
                                                                 (const float*)B.L.ptr, (float*)B.rgb.ptr);
    PBG_CUDA(cudaGetLastError());
    s->counters.kernel_launches += 1;
    cudaEventRecord(e1, st);
    PBG_CUDA(cudaMemcpyAsync(rgb_host, B.rgb.ptr, npix * 12, cudaMemcpyDeviceToHost, st));
    int rstat[4] = {0, 0, 0, 0};
    PBG_CUDA(cudaMemcpyAsync(rstat, B.rstat.ptr, 16, cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    stt.ms_total = ms;
    if (stats) *stats = stt;
    if (rstat[0] != 0) {
        char buf[200];
        snprintf(buf, sizeof(buf),
                 "pbg_render_stream: %d path vertices sampled a direction the BSDF rejects; the reference traces "
                 "such a ray again unchanged, so the stream no longer matches it",
                 rstat[0]);
        set_last_error(buf);
        return PBG_ERR_UNSUPPORTED;
    }
    return check_device_status(s, st);
}

}  // namespace pbg

extern "C" int pbg_render(pbg_scene* scene, const pbg_camera* camera, const pbg_light* lights,
                          int32_t nlights, const pbg_render_params* params, float* rgb,
                          pbg_render_stats* stats) {
    if (!scene) {
        pbg::set_last_error("pbg_render: scene is NULL");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(scene->device);
    return pbg::render(scene, camera, lights, nlights, params, nullptr, rgb, stats);
}

extern "C" int pbg_render_stream(pbg_scene* scene, const pbg_camera* camera, const pbg_light* lights,
                                 int32_t nlights, const pbg_render_params* params,
                                 const pbg_sample_stream* stream, float* rgb, pbg_render_stats* stats) {
    if (!scene || !stream) {
        pbg::set_last_error("pbg_render_stream: scene or stream is NULL");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(scene->device);
    return pbg::render(scene, camera, lights, nlights, params, stream, rgb, stats);
}
