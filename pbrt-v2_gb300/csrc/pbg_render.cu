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
//              (lights/point.cpp, a parallelogram area light), pbrt's
//              EstimateDirect weights (core/integrator.cpp:212-298), one
//              shadow slot per light sample and one bounce slot per path;
//   compact    slots -> dense queues, order-preserving: per-warp ballots give
//              ranks inside a block, a block scan gives block offsets;
//   resolve    unoccluded shadow contributions added per sample in light
//              sample order (deterministic, no float atomics);
//   film       per pixel, samples in order, through XYZ as ImageFilm does
//              (film/image.cpp AddSample / WriteImage), box filter.
//
// Random numbers: a counter-based hash of (seed, sample, dimension) -- not
// pbrt's MT19937 streams -- identical on every run and in the oracle's
// restatement.
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
// Russian roulette at 13, BSDF sample at 14-15.
__device__ __forceinline__ uint32_t dim_of(int bounce, int k) { return 2u + 16u * (uint32_t)bounce + (uint32_t)k; }
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
};

struct RenderConst {
    float r2c[16], c2w[16];
    int xres, yres, spp_x, spp_y, spp, jitter, max_depth, integrator;
    uint64_t seed;
    float albedo[3];
    int nlights;
    DevLight lights[4];
};

__global__ void raygen_kernel(RenderConst rc, int64_t n, float4* __restrict__ o4, float4* __restrict__ d4,
                              int32_t* __restrict__ qidx, float* __restrict__ L, float* __restrict__ beta) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int64_t pix = s / rc.spp;
    const int k = (int)(s % rc.spp);
    const int px = (int)(pix % rc.xres), py = (int)(pix / rc.xres);
    const int sx = k % rc.spp_x, sy = k / rc.spp_x;
    const float jx = rc.jitter ? rnd(rc.seed, (uint64_t)s, 0) : 0.5f;
    const float jy = rc.jitter ? rnd(rc.seed, (uint64_t)s, 1) : 0.5f;
    // (x + jx) * dx + xPos (samplers/stratified.cpp, StratifiedSample2D)
    const float ix = __fadd_rn(__fmul_rn(__fadd_rn((float)sx, jx), __frcp_rn((float)rc.spp_x)), (float)px);
    const float iy = __fadd_rn(__fmul_rn(__fadd_rn((float)sy, jy), __frcp_rn((float)rc.spp_y)), (float)py);
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

// Light sample j of light l at p: wi, radiance, pdf, shadow segment.
__device__ __forceinline__ bool sample_light(const DevLight& lt, V3 p, float eps, float u1, float u2,
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
    // VisibilityTester::SetSegment (core/light.h:79-84)
    const float dist = vlen(vsub(p, target));
    const V3 dn = vmul(vsub(target, p), __frcp_rn(dist));
    *so = make_float4(p.x, p.y, p.z, eps);
    *sd = make_float4(dn.x, dn.y, dn.z, __fmul_rn(dist, __fsub_rn(1.f, eps2)));
    return true;
}

// One queue entry: shade the hit, fill its shadow slots and its bounce slot.
__global__ void shade_kernel(RenderConst rc, int bounce, int64_t nq, const int32_t* __restrict__ qidx,
                             const float4* __restrict__ qo, const float4* __restrict__ qd,
                             const int32_t* __restrict__ prim, const float* __restrict__ th,
                             const float* __restrict__ b1v, const float* __restrict__ b2v,
                             const float* __restrict__ tri9, const float* __restrict__ uv6,
                             float* __restrict__ beta, int kslots, float4* __restrict__ so,
                             float4* __restrict__ sd, float* __restrict__ scontrib,
                             uint8_t* __restrict__ sflag, float4* __restrict__ no,
                             float4* __restrict__ nd_, uint8_t* __restrict__ nflag) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    for (int k = 0; k < kslots; ++k) sflag[j * kslots + k] = 0;
    nflag[j] = 0;
    const int32_t pr = prim[j];
    if (pr < 0) return;  // miss: no environment light
    const int64_t s = qidx[j];
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
    const V3 R = v3(rc.albedo[0], rc.albedo[1], rc.albedo[2]);
    const V3 fR = v3(__fmul_rn(R.x, kInvPi), __fmul_rn(R.y, kInvPi), __fmul_rn(R.z, kInvPi));
    const V3 bt = v3(beta[3 * s], beta[3 * s + 1], beta[3 * s + 2]);
    const float won = vdot(wo, ng);
    const V3 wol = fr.to_local(wo);

    // Direct lighting: every light and sample (directlighting) or one light
    // sample (path), core/integrator.cpp:73-176.
    const bool all = rc.integrator == PBG_INTEGRATOR_DIRECT;
    int slot = 0;
    for (int l = 0; l < rc.nlights; ++l) {
        const DevLight& lt = rc.lights[l];
        const int ns = all ? (lt.type == PBG_LIGHT_POINT ? 1 : max(lt.nsamples, 1)) : 1;
        if (!all && l > 0) break;  // UniformSampleOneLight: one light per vertex
        for (int q = 0; q < ns; ++q, ++slot) {
            const float u1 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, 2 * q) + 0);
            const float u2 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, 2 * q) + 1);
            V3 wi, Li;
            float pdf;
            float4 o_, d_;
            if (slot >= kslots) break;
            if (!sample_light(lt, g.p, eps, u1, u2, &wi, &Li, &pdf, &o_, &d_)) continue;
            if (!(pdf > 0.f) || (Li.x == 0.f && Li.y == 0.f && Li.z == 0.f)) continue;
            const bool refl = __fmul_rn(vdot(wi, ng), won) > 0.f;
            if (!refl) continue;  // f = 0: Lambertian reflects only
            const float absdot = fabsf(vdot(wi, fr.nn));
            V3 c;
            if (lt.type == PBG_LIGHT_POINT) {
                const float w = __fdiv_rn(absdot, pdf);
                c = v3(__fmul_rn(__fmul_rn(fR.x, Li.x), w), __fmul_rn(__fmul_rn(fR.y, Li.y), w),
                       __fmul_rn(__fmul_rn(fR.z, Li.z), w));
            } else {
                const V3 wil = fr.to_local(wi);
                const bool same = __fmul_rn(wol.z, wil.z) > 0.f;
                const float bpdf = same ? __fmul_rn(fabsf(wil.z), kInvPi) : 0.f;
                // PowerHeuristic(1, pdf, 1, bpdf)
                const float f2 = __fmul_rn(pdf, pdf), g2 = __fmul_rn(bpdf, bpdf);
                const float weight = __fdiv_rn(f2, __fadd_rn(f2, g2));
                const float w = __fdiv_rn(__fmul_rn(absdot, weight), pdf);
                c = v3(__fmul_rn(__fmul_rn(fR.x, Li.x), w), __fmul_rn(__fmul_rn(fR.y, Li.y), w),
                       __fmul_rn(__fmul_rn(fR.z, Li.z), w));
            }
            if (!all) {  // UniformSampleOneLight: times nLights, then the throughput
                const float fl = (float)rc.nlights;
                c = v3(__fmul_rn(c.x, fl), __fmul_rn(c.y, fl), __fmul_rn(c.z, fl));
                c = v3(__fmul_rn(bt.x, c.x), __fmul_rn(bt.y, c.y), __fmul_rn(bt.z, c.z));
            }
            // (directlighting divides each light's visible sum by nSamples
            // when the shadow results are resolved)
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
    const float u1 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, kDimBsdf));
    const float u2 = rnd(rc.seed, (uint64_t)s, dim_of(bounce, kDimBsdf + 1));
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
        theta = __fmul_rn(theta, 0.785398163397448309616f);
        float st, ct;
        own_sincos(theta, &st, &ct);
        dx = __fmul_rn(r, ct);
        dy = __fmul_rn(r, st);
    }
    V3 wil = v3(dx, dy, __fsqrt_rn(fmaxf(0.f, __fsub_rn(__fsub_rn(1.f, __fmul_rn(dx, dx)), __fmul_rn(dy, dy)))));
    if (wol.z < 0.f) wil.z = -wil.z;
    const bool same = __fmul_rn(wol.z, wil.z) > 0.f;
    const float pdf = same ? __fmul_rn(fabsf(wil.z), kInvPi) : 0.f;
    const V3 wi = fr.to_world(wil);
    const bool refl = __fmul_rn(vdot(wi, ng), won) > 0.f;
    if (!refl || !(pdf > 0.f)) return;
    const float absdot = fabsf(vdot(wi, fr.nn));
    // pathThroughput *= f * AbsDot(wi, n) / pdf
    V3 nb = v3(__fmul_rn(bt.x, __fdiv_rn(__fmul_rn(fR.x, absdot), pdf)),
               __fmul_rn(bt.y, __fdiv_rn(__fmul_rn(fR.y, absdot), pdf)),
               __fmul_rn(bt.z, __fdiv_rn(__fmul_rn(fR.z, absdot), pdf)));
    if (bounce > 3) {  // Russian roulette (integrators/path.cpp:117-124)
        const float y = __fadd_rn(__fadd_rn(__fmul_rn(0.212671f, nb.x), __fmul_rn(0.715160f, nb.y)),
                                  __fmul_rn(0.072169f, nb.z));
        const float cont = fminf(0.5f, y);
        if (rnd(rc.seed, (uint64_t)s, dim_of(bounce, kDimRR)) > cont) return;
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

// Unoccluded shadow contributions, added per entry in slot order.
// directlighting: per light, Ld = sum of its visible samples, L += Ld / ns
// (UniformSampleAllLights, core/integrator.cpp:73-122); path: the single
// slot already carries beta * nLights * Ld.
__global__ void resolve_kernel(RenderConst rc, int64_t nq, int kslots, const int32_t* __restrict__ qidx,
                               const uint8_t* __restrict__ sflag, const int32_t* __restrict__ spos,
                               const uint8_t* __restrict__ occ, const float* __restrict__ scontrib,
                               float* __restrict__ L) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    const int64_t s = qidx[j];
    float lx = L[3 * s], ly = L[3 * s + 1], lz = L[3 * s + 2];
    if (rc.integrator == PBG_INTEGRATOR_DIRECT) {
        int k = 0;
        for (int l = 0; l < rc.nlights; ++l) {
            const int ns = rc.lights[l].type == PBG_LIGHT_POINT ? 1 : max(rc.lights[l].nsamples, 1);
            float ax = 0.f, ay = 0.f, az = 0.f;
            for (int q = 0; q < ns && k < kslots; ++q, ++k) {
                const int64_t si = j * kslots + k;
                if (!sflag[si] || occ[spos[si]]) continue;
                ax = __fadd_rn(ax, scontrib[3 * si]);
                ay = __fadd_rn(ay, scontrib[3 * si + 1]);
                az = __fadd_rn(az, scontrib[3 * si + 2]);
            }
            const float fn = (float)ns;
            lx = __fadd_rn(lx, __fdiv_rn(ax, fn));
            ly = __fadd_rn(ly, __fdiv_rn(ay, fn));
            lz = __fadd_rn(lz, __fdiv_rn(az, fn));
        }
    } else {
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
// divided by the weight sum, clamped at zero (film/image.cpp).
__global__ void film_kernel(int64_t npix, int spp, const float* __restrict__ L, float* __restrict__ rgb) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float X = 0.f, Y = 0.f, Z = 0.f, w = 0.f;
    for (int k = 0; k < spp; ++k) {
        const int64_t s = p * spp + k;
        const float r = L[3 * s], g = L[3 * s + 1], b = L[3 * s + 2];
        const float x = __fadd_rn(__fadd_rn(__fmul_rn(0.412453f, r), __fmul_rn(0.357580f, g)), __fmul_rn(0.180423f, b));
        const float y = __fadd_rn(__fadd_rn(__fmul_rn(0.212671f, r), __fmul_rn(0.715160f, g)), __fmul_rn(0.072169f, b));
        const float z = __fadd_rn(__fadd_rn(__fmul_rn(0.019334f, r), __fmul_rn(0.119193f, g)), __fmul_rn(0.950227f, b));
        X = __fadd_rn(X, x);
        Y = __fadd_rn(Y, y);
        Z = __fadd_rn(Z, z);
        w = __fadd_rn(w, 1.f);
    }
    const float R = __fsub_rn(__fsub_rn(__fmul_rn(3.240479f, X), __fmul_rn(1.537150f, Y)), __fmul_rn(0.498535f, Z));
    const float G = __fadd_rn(__fadd_rn(__fmul_rn(-0.969256f, X), __fmul_rn(1.875991f, Y)), __fmul_rn(0.041556f, Z));
    const float B = __fadd_rn(__fsub_rn(__fmul_rn(0.055648f, X), __fmul_rn(0.204043f, Y)), __fmul_rn(1.057311f, Z));
    const float inv = __frcp_rn(w);
    rgb[3 * p] = fmaxf(0.f, __fmul_rn(R, inv));
    rgb[3 * p + 1] = fmaxf(0.f, __fmul_rn(G, inv));
    rgb[3 * p + 2] = fmaxf(0.f, __fmul_rn(B, inv));
}

// ------------------------------------------------------------------ host

int scan_counts(pbg_scene* s, uint32_t* a, int64_t m, cudaStream_t st);

struct RenderBuffers {
    DeviceBuffer o4, d4, qidx, L, beta, prim, t, b1, b2, so, sd, scontrib, sflag, spos, sqo, sqd, occ,
        no, nd, nflag, qidx2, o42, d42, counts, rgb;
    ~RenderBuffers() {
        DeviceBuffer* all[] = {&o4, &d4, &qidx, &L, &beta, &prim, &t, &b1, &b2, &so, &sd, &scontrib,
                               &sflag, &spos, &sqo, &sqd, &occ, &no, &nd, &nflag, &qidx2, &o42, &d42,
                               &counts, &rgb};
        for (DeviceBuffer* b : all) release(*b);
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

int render(pbg_scene* s, const pbg_camera* cam, const pbg_light* lights, int32_t nlights,
           const pbg_render_params* prm, float* rgb_host, pbg_render_stats* stats) {
    if (!cam || !prm || nlights < 0 || nlights > 4 || (nlights > 0 && !lights) || !rgb_host ||
        cam->xres <= 0 || cam->yres <= 0 || prm->spp_x <= 0 || prm->spp_y <= 0) {
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
    for (int k = 0; k < 3; ++k) rc.albedo[k] = prm->albedo[k];
    rc.nlights = nlights;
    int kslots = 0;
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
    const int64_t n = npix * rc.spp;
    if (n > (int64_t)INT32_MAX / std::max(kslots, 1)) {
        set_last_error("pbg_render: image too large for one batch");
        return PBG_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t st = s->stream;
    if (!s->render_bufs) s->render_bufs = new RenderBuffers();
    RenderBuffers& B = *s->render_bufs;  // grown on demand, kept for the next frame
    int r;
    const size_t nk = (size_t)n * kslots;
    if ((r = ensure(B.o4, n * 16)) || (r = ensure(B.d4, n * 16)) || (r = ensure(B.qidx, n * 4)) ||
        (r = ensure(B.L, n * 12)) || (r = ensure(B.beta, n * 12)) || (r = ensure(B.prim, n * 4)) ||
        (r = ensure(B.t, n * 4)) || (r = ensure(B.b1, n * 4)) || (r = ensure(B.b2, n * 4)) ||
        (r = ensure(B.so, nk * 16)) || (r = ensure(B.sd, nk * 16)) || (r = ensure(B.scontrib, nk * 12)) ||
        (r = ensure(B.sflag, nk)) || (r = ensure(B.spos, nk * 4)) || (r = ensure(B.sqo, nk * 16)) ||
        (r = ensure(B.sqd, nk * 16)) || (r = ensure(B.occ, nk)) || (r = ensure(B.no, n * 16)) ||
        (r = ensure(B.nd, n * 16)) || (r = ensure(B.nflag, n)) || (r = ensure(B.qidx2, n * 4)) ||
        (r = ensure(B.o42, n * 16)) || (r = ensure(B.d42, n * 16)) ||
        (r = ensure(B.counts, ((nk + 255) / 256 + 64) * 4 + 4096)) || (r = ensure(B.rgb, npix * 12)))
        return r;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    raygen_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        rc, n, (float4*)B.o4.ptr, (float4*)B.d4.ptr, (int32_t*)B.qidx.ptr, (float*)B.L.ptr,
        (float*)B.beta.ptr);
    PBG_CUDA(cudaGetLastError());
    s->counters.kernel_launches += 1;
    pbg_render_stats stt{};
    stt.camera_rays = (uint64_t)n;
    int64_t nq = n;
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
    for (int bounce = 0; nq > 0; ++bounce) {
        s->walk_hint = bounce > 0 ? 1 : 0;
        if ((r = pbg_intersect_device(s, (const float*)qo, (const float*)qd, nullptr, nq,
                                      (int32_t*)B.prim.ptr, (float*)B.t.ptr, (float*)B.b1.ptr,
                                      (float*)B.b2.ptr, st)))
            return r;
        stt.nearest_rays += (uint64_t)nq;
        const int64_t nslots = nq * kslots;
        shade_kernel<<<(unsigned)((nq + 127) / 128), 128, 0, st>>>(
            rc, bounce, nq, qi, qo, qd, (const int32_t*)B.prim.ptr, (const float*)B.t.ptr,
            (const float*)B.b1.ptr, (const float*)B.b2.ptr, (const float*)s->tri9.ptr,
            (const float*)s->uv6.ptr, (float*)B.beta.ptr, kslots, (float4*)B.so.ptr, (float4*)B.sd.ptr,
            (float*)B.scontrib.ptr, (uint8_t*)B.sflag.ptr, (float4*)B.no.ptr, (float4*)B.nd.ptr,
            (uint8_t*)B.nflag.ptr);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 1;
        // shadow queue
        int64_t nsh = 0;
        if ((r = compact_count(s, (const uint8_t*)B.sflag.ptr, nslots, (uint32_t*)B.counts.ptr, &nsh, st)))
            return r;
        compact_shadow_kernel<<<(unsigned)((nslots + 255) / 256), 256, 0, st>>>(
            (const uint8_t*)B.sflag.ptr, nslots, (const uint32_t*)B.counts.ptr, (const float4*)B.so.ptr,
            (const float4*)B.sd.ptr, (float4*)B.sqo.ptr, (float4*)B.sqd.ptr, (int32_t*)B.spos.ptr);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 1;
        if (nsh > 0 && (r = pbg_occluded_device(s, (const float*)B.sqo.ptr, (const float*)B.sqd.ptr,
                                                nullptr, nsh, (uint8_t*)B.occ.ptr, st)))
            return r;
        stt.shadow_rays += (uint64_t)nsh;
        resolve_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(
            rc, nq, kslots, qi, (const uint8_t*)B.sflag.ptr, (const int32_t*)B.spos.ptr,
            (const uint8_t*)B.occ.ptr, (const float*)B.scontrib.ptr, (float*)B.L.ptr);
        PBG_CUDA(cudaGetLastError());
        s->counters.kernel_launches += 1;
        if (rc.integrator != PBG_INTEGRATOR_PATH) break;
        // bounce queue
        int64_t nn = 0;
        if ((r = compact_count(s, (const uint8_t*)B.nflag.ptr, nq, (uint32_t*)B.counts.ptr, &nn, st)))
            return r;
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
    // online training of the learned ordering on this frame's records
    if (s->learn && s->learn->enabled && (r = learn_train(s, 0, st))) return r;
    film_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(npix, rc.spp, (const float*)B.L.ptr,
                                                                 (float*)B.rgb.ptr);
    PBG_CUDA(cudaGetLastError());
    s->counters.kernel_launches += 1;
    cudaEventRecord(e1, st);
    PBG_CUDA(cudaMemcpyAsync(rgb_host, B.rgb.ptr, npix * 12, cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    stt.ms_total = ms;
    if (stats) *stats = stt;
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
    return pbg::render(scene, camera, lights, nlights, params, rgb, stats);
}
