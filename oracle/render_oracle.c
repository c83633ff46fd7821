/*
 * render_oracle.c -- CPU restatement of the breadth-first renderer's image
 * for the GPU wavefront to be checked against.
 *
 * TEST INFRASTRUCTURE ONLY (loaded by tests/ and bench.py's CPU leg).
 *
 * One sample at a time, depth first, in the shape of pbrt's single-ray
 * integrators:
 *   camera      cameras/perspective.cpp GenerateRayDifferential with the
 *               caller's RasterToCamera / CameraToWorld matrices,
 *               stratified image samples (samplers/stratified.cpp)
 *   direct      integrators/directlighting.cpp + UniformSampleAllLights and
 *               EstimateDirect, core/integrator.cpp:73-122, :212-298
 *   path        integrators/path.cpp:43-157 (UniformSampleOneLight, cosine
 *               BSDF sampling, Russian roulette after bounce 3); the
 *               BSDF-sampled half of EstimateDirect traces no ray, as in the
 *               fork's batch path (core/integrator.cpp:431-435)
 *   materials   MatteMaterial with sigma 0 -> Lambertian (core/reflection.cpp)
 *   lights      PointLight (lights/point.cpp); a one-sided parallelogram
 *               emitter sampled uniformly by area
 *   film        ImageFilm: RGB -> XYZ per sample, box filter, XYZ -> RGB
 *               (film/image.cpp, core/spectrum.h:43-54)
 * Random numbers come from a counter-based hash of (seed, sample,
 * dimension): the same stream the GPU renderer draws, not pbrt's MT19937.
 * Intersections use the oracle's BVH, whose answers equal pbrt's in-order
 * triangle loop.  Build with -ffp-contract=off.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

void* orc_bvh_build(const float* tris, int64_t ntri, int maxprims);
void orc_bvh_free(void* p);
int32_t orc_bvh_trace(void* bvh, const float o[3], const float d[3], float mint, float maxt,
                      int anyhit, float* t, float* b1, float* b2);
void orc_hit_geometry(const float* tri, const float* uv6, const float o[3], const float d[3],
                      float t, float b1, float b2, float* out);

#define INV_PI 0.31830988618379067154f

typedef struct {
    float r2c[16], c2w[16];
    int xres, yres;
} orc_camera;

typedef struct {
    int type, nsamples;
    float pos[3], I[3], quad[12], L[3];
} orc_light;

typedef struct {
    int integrator, spp_x, spp_y, jitter, max_depth;
    uint64_t seed;
    float albedo[3];
} orc_params;

/* splitmix64 finalizer */
static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static float rnd(uint64_t seed, uint64_t sample, uint32_t dim) {
    uint64_t h = mix64(seed ^ mix64(sample * 0x100000001B3ull + dim));
    return (float)(h >> 40) * 0x1p-24f;
}
static uint32_t dim_of(int bounce, int k) { return 2u + 16u * (uint32_t)bounce + (uint32_t)k; }

/* sin and cos in float from the Cephes single-precision polynomials
 * (S. Moshier, Cephes Math Library, sinf.c/cosf.c coefficients) after a
 * two-constant Cody-Waite reduction by pi/2; the GPU renderer evaluates the
 * same operations in the same order, so both give identical bits. */
static void own_sincos(float a, float* s, float* c) {
    float jf = rintf(a * 0.636619772367581343f);
    int j = (int)jf;
    float r = (a - jf * 1.5703125f) - jf * 4.83826794897e-4f;
    float z = r * r;
    float sp = ((-1.9515295891e-4f * z + 8.3321608736e-3f) * z - 1.6666654611e-1f) * z * r + r;
    float cp = ((2.443315711809948e-5f * z - 1.388731625493765e-3f) * z + 4.166664568298827e-2f) * z * z
               - 0.5f * z + 1.f;
    switch (j & 3) {
        case 0: *s = sp; *c = cp; break;
        case 1: *s = cp; *c = -sp; break;
        case 2: *s = -sp; *c = -cp; break;
        default: *s = -cp; *c = sp; break;
    }
}

typedef struct { float x, y, z; } vec;
static vec V(float x, float y, float z) { vec v = {x, y, z}; return v; }
static vec sub(vec a, vec b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static vec add(vec a, vec b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static vec scl(vec a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static float dot(vec a, vec b) { float s = a.x * b.x + a.y * b.y; return s + a.z * b.z; }
static vec cross(vec a, vec b) {
    double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return V((float)((ay * bz) - (az * by)), (float)((az * bx) - (ax * bz)), (float)((ax * by) - (ay * bx)));
}
static float length(vec a) { return sqrtf(dot(a, a)); }
static vec normalize(vec a) { float inv = 1.f / length(a); return scl(a, inv); }

static vec xpoint(const float* m, vec p) {
    float xp = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
    float yp = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    float zp = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
    float wp = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    if (wp == 1.f) return V(xp, yp, zp);
    float inv = 1.f / wp;
    return V(inv * xp, inv * yp, inv * zp);
}
static vec xvector(const float* m, vec v) {
    return V(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
             m[8] * v.x + m[9] * v.y + m[10] * v.z);
}

typedef struct {
    const float* tris;
    void* bvh;
    const orc_camera* cam;
    const orc_light* lights;
    int nlights;
    const orc_params* prm;
    float* L; /* [n][3] per sample (NULL: counting only) */
    int64_t begin, end;   /* sample slots [begin, end) ... */
    int64_t stride, first; /* ... are samples first + slot * stride */
    uint64_t nearest, shadow; /* rays traced by this job */
} job_t;

static int occluded(job_t* j, vec o, vec d, float mint, float maxt) {
    float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    j->shadow++;
    return orc_bvh_trace(j->bvh, oo, dd, mint, maxt, 1, NULL, NULL, NULL) >= 0;
}

/* EstimateDirect for one light sample (u1, u2); 0 if occluded or black. */
static vec estimate_direct(job_t* j, const orc_light* lt, vec p, float eps, vec nn, vec ng,
                           vec wo, const vec fr[3], vec fR, float u1, float u2) {
    vec zero = V(0.f, 0.f, 0.f);
    vec target, wi, Li;
    float pdf, eps2;
    if (lt->type == 0) {
        target = V(lt->pos[0], lt->pos[1], lt->pos[2]);
        wi = normalize(sub(target, p));
        pdf = 1.f;
        vec dv = sub(target, p);
        float d2 = dot(dv, dv);
        Li = V(lt->I[0] / d2, lt->I[1] / d2, lt->I[2] / d2);
        eps2 = 0.f;
    } else {
        vec q0 = V(lt->quad[0], lt->quad[1], lt->quad[2]);
        vec e1 = V(lt->quad[3] - lt->quad[0], lt->quad[4] - lt->quad[1], lt->quad[5] - lt->quad[2]);
        vec e3 = V(lt->quad[9] - lt->quad[0], lt->quad[10] - lt->quad[1], lt->quad[11] - lt->quad[2]);
        double cx = (double)e1.y * e3.z - (double)e1.z * e3.y;
        double cy = (double)e1.z * e3.x - (double)e1.x * e3.z;
        double cz = (double)e1.x * e3.y - (double)e1.y * e3.x;
        double len = sqrt(cx * cx + cy * cy + cz * cz);
        float area = (float)len;
        vec n = V(len > 0 ? (float)(cx / len) : 0.f, len > 0 ? (float)(cy / len) : 0.f,
                  len > 0 ? (float)(cz / len) : 0.f);
        target = add(add(q0, scl(e1, u1)), scl(e3, u2));
        vec dv = sub(target, p);
        wi = normalize(dv);
        float d2 = dot(dv, dv);
        float cosl = -dot(n, wi);
        if (!(cosl > 0.f) || !(d2 > 0.f)) return zero;
        pdf = d2 / (cosl * area);
        Li = V(lt->L[0], lt->L[1], lt->L[2]);
        eps2 = 1e-3f;
    }
    if (!(pdf > 0.f) || (Li.x == 0.f && Li.y == 0.f && Li.z == 0.f)) return zero;
    if (!(dot(wi, ng) * dot(wo, ng) > 0.f)) return zero; /* BSDF::f: reflection only */
    /* VisibilityTester::SetSegment */
    float dist = length(sub(p, target));
    vec dn = scl(sub(target, p), 1.f / dist);
    if (occluded(j, p, dn, eps, dist * (1.f - eps2))) return zero;
    float absdot = fabsf(dot(wi, nn));
    float w;
    if (lt->type == 0) {
        w = absdot / pdf;
    } else {
        vec wol = V(dot(wo, fr[0]), dot(wo, fr[1]), dot(wo, fr[2]));
        vec wil = V(dot(wi, fr[0]), dot(wi, fr[1]), dot(wi, fr[2]));
        float bpdf = (wol.z * wil.z > 0.f) ? fabsf(wil.z) * INV_PI : 0.f;
        float f2 = pdf * pdf, g2 = bpdf * bpdf;
        float weight = f2 / (f2 + g2);
        w = (absdot * weight) / pdf;
    }
    return V((fR.x * Li.x) * w, (fR.y * Li.y) * w, (fR.z * Li.z) * w);
}

static void* render_worker(void* arg) {
    job_t* j = (job_t*)arg;
    const orc_camera* cam = j->cam;
    const orc_params* prm = j->prm;
    const int spp = prm->spp_x * prm->spp_y;
    const vec fR = V(prm->albedo[0] * INV_PI, prm->albedo[1] * INV_PI, prm->albedo[2] * INV_PI);
    for (int64_t slot = j->begin; slot < j->end; ++slot) {
        const int64_t s = j->first + slot * j->stride;
        int64_t pix = s / spp;
        int k = (int)(s % spp);
        int px = (int)(pix % cam->xres), py = (int)(pix / cam->xres);
        int sx = k % prm->spp_x, sy = k / prm->spp_x;
        float jx = prm->jitter ? rnd(prm->seed, (uint64_t)s, 0) : 0.5f;
        float jy = prm->jitter ? rnd(prm->seed, (uint64_t)s, 1) : 0.5f;
        float ix = ((float)sx + jx) * (1.f / (float)prm->spp_x) + (float)px;
        float iy = ((float)sy + jy) * (1.f / (float)prm->spp_y) + (float)py;
        vec pc = xpoint(cam->r2c, V(ix, iy, 0.f));
        vec o = xpoint(cam->c2w, V(0.f, 0.f, 0.f));
        vec d = xvector(cam->c2w, normalize(pc));
        float mint = 0.f;
        vec L = V(0.f, 0.f, 0.f), beta = V(1.f, 1.f, 1.f);
        int max_depth = prm->max_depth > 0 ? prm->max_depth : 5;
        for (int bounce = 0;; ++bounce) {
            float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
            float t, b1, b2;
            int32_t prim = orc_bvh_trace(j->bvh, oo, dd, mint, INFINITY, 0, &t, &b1, &b2);
            j->nearest++;
            if (prim < 0) break;
            float g[14];
            orc_hit_geometry(j->tris + 9 * (int64_t)prim, NULL, oo, dd, t, b1, b2, g);
            vec p = V(g[0], g[1], g[2]);
            vec dpdu = V(g[3], g[4], g[5]);
            vec nn = V(g[9], g[10], g[11]);
            float eps = 1e-3f * t;
            vec fr[3];
            fr[0] = normalize(dpdu);     /* sn */
            fr[1] = cross(nn, fr[0]);    /* tn */
            fr[2] = nn;
            vec wo = V(-d.x, -d.y, -d.z);
            if (prm->integrator == 0) {
                for (int l = 0; l < j->nlights; ++l) {
                    const orc_light* lt = &j->lights[l];
                    int ns = lt->type == 0 ? 1 : (lt->nsamples > 0 ? lt->nsamples : 1);
                    vec Ld = V(0.f, 0.f, 0.f);
                    for (int q = 0; q < ns; ++q) {
                        float u1 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 2 * q));
                        float u2 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 2 * q) + 1);
                        Ld = add(Ld, estimate_direct(j, lt, p, eps, nn, nn, wo, fr, fR, u1, u2));
                    }
                    float fn = (float)ns;
                    L = add(L, V(Ld.x / fn, Ld.y / fn, Ld.z / fn));
                }
                break;
            }
            if (j->nlights > 0) {
                float u1 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 0));
                float u2 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 1));
                vec e = estimate_direct(j, &j->lights[0], p, eps, nn, nn, wo, fr, fR, u1, u2);
                float fl = (float)j->nlights;
                e = V(e.x * fl, e.y * fl, e.z * fl);
                L = add(L, V(beta.x * e.x, beta.y * e.y, beta.z * e.z));
            }
            /* cosine-weighted BSDF sample (ConcentricSampleDisk) */
            float u1 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 14));
            float u2 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 15));
            float sxd = 2.f * u1 - 1.f, syd = 2.f * u2 - 1.f, dx = 0.f, dy = 0.f;
            if (!(sxd == 0.f && syd == 0.f)) {
                float r, theta;
                if (sxd >= -syd) {
                    if (sxd > syd) { r = sxd; theta = syd > 0.f ? syd / r : 8.f + syd / r; }
                    else { r = syd; theta = 2.f - sxd / r; }
                } else {
                    if (sxd <= syd) { r = -sxd; theta = 4.f - syd / r; }
                    else { r = -syd; theta = 6.f + sxd / r; }
                }
                theta *= 0.785398163397448309616f;
                float st, ct;
                own_sincos(theta, &st, &ct);
                dx = r * ct;
                dy = r * st;
            }
            vec wil = V(dx, dy, sqrtf(fmaxf(0.f, 1.f - dx * dx - dy * dy)));
            vec wol = V(dot(wo, fr[0]), dot(wo, fr[1]), dot(wo, fr[2]));
            if (wol.z < 0.f) wil.z = -wil.z;
            float pdf = (wol.z * wil.z > 0.f) ? fabsf(wil.z) * INV_PI : 0.f;
            vec wi = V(fr[0].x * wil.x + fr[1].x * wil.y + fr[2].x * wil.z,
                       fr[0].y * wil.x + fr[1].y * wil.y + fr[2].y * wil.z,
                       fr[0].z * wil.x + fr[1].z * wil.y + fr[2].z * wil.z);
            if (!(dot(wi, nn) * dot(wo, nn) > 0.f) || !(pdf > 0.f)) break;
            float absdot = fabsf(dot(wi, nn));
            beta = V(beta.x * ((fR.x * absdot) / pdf), beta.y * ((fR.y * absdot) / pdf),
                     beta.z * ((fR.z * absdot) / pdf));
            if (bounce > 3) {
                float y = 0.212671f * beta.x + 0.715160f * beta.y + 0.072169f * beta.z;
                float cont = fminf(0.5f, y);
                if (rnd(prm->seed, (uint64_t)s, dim_of(bounce, 13)) > cont) break;
                beta = V(beta.x / cont, beta.y / cont, beta.z / cont);
            }
            if (bounce == max_depth) break;
            o = p;
            d = wi;
            mint = eps;
        }
        if (j->L) {
            j->L[3 * s] = L.x;
            j->L[3 * s + 1] = L.y;
            j->L[3 * s + 2] = L.z;
        }
    }
    return NULL;
}

/* Runs nslots samples (first + k * stride, k < nslots) on nthreads threads
 * over a prebuilt BVH; out receives the radiance when non-NULL (indexed by
 * sample), counts[0] / counts[1] the nearest-hit and shadow rays traced. */
static void run_samples(const float* tris, void* bvh, const orc_camera* cam, const orc_light* lights,
                        int nlights, const orc_params* prm, float* L, int64_t first, int64_t stride,
                        int64_t nslots, int nthreads, uint64_t counts[2]) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    job_t jobs[256];
    pthread_t th[256];
    int64_t chunk = (nslots + nthreads - 1) / nthreads;
    int started = 0;
    for (int k = 0; k < nthreads; ++k) {
        job_t jb = {tris, bvh, cam, lights, nlights, prm, L, k * chunk,
                    (k + 1) * chunk < nslots ? (k + 1) * chunk : nslots, stride, first, 0, 0};
        jobs[k] = jb;
        if (jobs[k].begin >= jobs[k].end) break;
        pthread_create(&th[k], NULL, render_worker, &jobs[k]);
        started = k + 1;
    }
    counts[0] = counts[1] = 0;
    for (int k = 0; k < started; ++k) {
        pthread_join(th[k], NULL);
        counts[0] += jobs[k].nearest;
        counts[1] += jobs[k].shadow;
    }
}

/* The CPU baseline's bounded sample of a frame: the BVH is built once
 * (orc_render_bvh), then orc_render_count traces the samples first,
 * first + stride, ... of the image and returns only the ray counts. */
void* orc_render_bvh(const float* tris, int64_t ntri) { return orc_bvh_build(tris, ntri, 4); }
void orc_render_bvh_free(void* bvh) { orc_bvh_free(bvh); }
void orc_render_count(const float* tris, void* bvh, const orc_camera* cam, const orc_light* lights,
                      int nlights, const orc_params* prm, int64_t first, int64_t stride, int nthreads,
                      uint64_t* counts) {
    const int64_t n = (int64_t)cam->xres * cam->yres * prm->spp_x * prm->spp_y;
    if (stride < 1) stride = 1;
    const int64_t nslots = first < n ? (n - first + stride - 1) / stride : 0;
    run_samples(tris, bvh, cam, lights, nlights, prm, NULL, first, stride, nslots, nthreads, counts);
}

/* rgb: [yres][xres][3].  nthreads host threads over the samples. */
void orc_render(const float* tris, int64_t ntri, const orc_camera* cam, const orc_light* lights,
                int nlights, const orc_params* prm, float* rgb, int nthreads) {
    const int spp = prm->spp_x * prm->spp_y;
    const int64_t npix = (int64_t)cam->xres * cam->yres, n = npix * spp;
    float* L = (float*)malloc((size_t)(n > 0 ? n : 1) * 3 * sizeof(float));
    void* bvh = orc_bvh_build(tris, ntri, 4);
    uint64_t counts[2];
    run_samples(tris, bvh, cam, lights, nlights, prm, L, 0, 1, n, nthreads, counts);
    for (int64_t p = 0; p < npix; ++p) {
        float X = 0.f, Y = 0.f, Z = 0.f, w = 0.f;
        for (int k = 0; k < spp; ++k) {
            const float* l = L + 3 * (p * spp + k);
            float x = 0.412453f * l[0] + 0.357580f * l[1] + 0.180423f * l[2];
            float y = 0.212671f * l[0] + 0.715160f * l[1] + 0.072169f * l[2];
            float z = 0.019334f * l[0] + 0.119193f * l[1] + 0.950227f * l[2];
            X += x; Y += y; Z += z; w += 1.f;
        }
        float R = 3.240479f * X - 1.537150f * Y - 0.498535f * Z;
        float G = -0.969256f * X + 1.875991f * Y + 0.041556f * Z;
        float B = 0.055648f * X - 0.204043f * Y + 1.057311f * Z;
        float inv = 1.f / w;
        rgb[3 * p] = fmaxf(0.f, R * inv);
        rgb[3 * p + 1] = fmaxf(0.f, G * inv);
        rgb[3 * p + 2] = fmaxf(0.f, B * inv);
    }
    orc_bvh_free(bvh);
    free(L);
}
