/*
 * render_oracle.c -- CPU restatement of the breadth-first renderer's image
 * for the GPU wavefront to be checked against.
 *
 * TEST INFRASTRUCTURE ONLY (loaded by tests/ and bench.py's CPU leg).
 *
 * The structure of the reference's breadth-first renderer: the samples are
 * taken in tasks of at most 409,600 (renderers/breadth-first.cpp:18-97,
 * scene MaxRaysPerCall), and each task is one wavefront -- all camera rays
 * traced, all hits shaded, all bounce rays traced, ... -- as the batch
 * integrators do it:
 *   camera      cameras/perspective.cpp GenerateRayDifferential with the
 *               caller's RasterToCamera / CameraToWorld matrices,
 *               stratified image samples (samplers/stratified.cpp)
 *   direct      integrators/directlighting.cpp:112-133 with the batch
 *               UniformSampleAllLights / EstimateDirect
 *               (core/integrator.cpp:73-122, :358-455): every light sample's
 *               contribution summed (not divided by the sample count), then
 *               the emission of camera hits on emitters
 *   path        integrators/path.cpp:43-157 with the batch
 *               UniformSampleOneLight / EstimateDirect
 *               (core/integrator.cpp:125-176, :212-298), cosine BSDF
 *               sampling, Russian roulette after bounce 3
 *   materials   MatteMaterial with sigma 0 -> Lambertian (core/reflection.cpp)
 *   lights      PointLight (lights/point.cpp); DiffuseAreaLight on scene
 *               triangles (lights/diffuse.cpp:61-79, ShapeSet
 *               core/light.cpp:105-165, Shape::Pdf core/shape.cpp:78-91,
 *               Triangle::Sample / Area shapes/trianglemesh.cpp:276-282,
 *               :436-447); an emitter on a parallelogram sampled by area
 *   film        ImageFilm: RGB -> XYZ per sample, box filter footprint,
 *               XYZ -> RGB (film/image.cpp, core/spectrum.h:43-54); samples
 *               breadthFirst::Li rejects (NaN, negative or infinite
 *               luminance) add black
 * Random numbers: a counter-based hash of (seed, sample, dimension) -- the
 * stream the GPU renderer draws by default -- or the reference's own values
 * (orc_render_stream: one task's sampler output and RNG continuation,
 * consumed in the batch integrators' order).  Intersections use the
 * oracle's BVH, whose answers equal pbrt's in-order triangle loop.  Build
 * with -ffp-contract=off.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

void* orc_bvh_build(const float* tris, int64_t ntri, int maxprims);
void* orc_bvh_build_mode(const float* tris, int64_t ntri, int maxprims, int box_degenerate);
void orc_bvh_free(void* p);
int32_t orc_bvh_trace(void* bvh, const float o[3], const float d[3], float mint, float maxt,
                      int anyhit, float* t, float* b1, float* b2);
void orc_hit_geometry(const float* tri, const float* uv6, const float o[3], const float d[3],
                      float t, float b1, float b2, float* out);
int orc_tri_intersect(const float* tri, const float o[3], const float dir[3], float mint,
                      float maxt, float* t_out, float* b1_out, float* b2_out);

#define INV_PI 0.31830988618379067154f
#define TASK_SAMPLES 409600
#define PATH_SAMPLE_DEPTH 3

typedef struct {
    float r2c[16], c2w[16];
    int xres, yres;
} orc_camera;

typedef struct {
    int type, nsamples;
    float pos[3], I[3], quad[12], L[3];
    int first_tri, ntri;
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
static uint32_t dim_extra(int bounce, int k) { return 512u + 16u * (uint32_t)bounce + (uint32_t)k; }

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
static vec neg(vec a) { return V(-a.x, -a.y, -a.z); }
static float dot(vec a, vec b) { float s = a.x * b.x + a.y * b.y; return s + a.z * b.z; }
static vec cross(vec a, vec b) {
    double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return V((float)((ay * bz) - (az * by)), (float)((az * bx) - (ax * bz)), (float)((ax * by) - (ay * bx)));
}
static float length(vec a) { return sqrtf(dot(a, a)); }
static vec normalize(vec a) { float inv = 1.f / length(a); return scl(a, inv); }
static vec tri_vertex(const float* v9, int k) { return V(v9[3 * k], v9[3 * k + 1], v9[3 * k + 2]); }

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

/* ------------------------------------------------------------- the scene */

typedef struct {
    const float* tris;
    const float* uvs;
    void* bvh;
    const orc_camera* cam;
    const orc_light* lights;
    int nlights;
    const orc_params* prm;
    /* triangle emitters: areas[ntri], cdf[ntri + 1], total area, per light */
    float* etab[8];
    /* the reference's sample stream (NULL: the hash) */
    const float* s_img;
    const float* s_dims;
    int ndims;
    const float* s_rng;
    int64_t nrng;
} ctx_t;

/* ShapeSet's i-th shape: its constructor refines the mesh through a stack
 * (todo.back(), core/light.cpp:106-118), so the mesh's triangles come out
 * last first. */
static int64_t shape_tri(const orc_light* lt, int i) { return (int64_t)lt->first_tri + lt->ntri - 1 - i; }

/* Triangle::Area, the ShapeSet's total area and its Distribution1D CDF,
 * in shape order. */
static float* emitter_table(const float* tris, const orc_light* lt) {
    int n = lt->ntri;
    float* tab = (float*)malloc(sizeof(float) * (2 * n + 2));
    float sum = 0.f;
    for (int i = 0; i < n; ++i) {
        const float* v = tris + 9 * shape_tri(lt, i);
        vec p1 = tri_vertex(v, 0);
        float a = 0.5f * length(cross(sub(tri_vertex(v, 1), p1), sub(tri_vertex(v, 2), p1)));
        tab[i] = a;
        sum += a;
    }
    float* cdf = tab + n;
    cdf[0] = 0.f;
    for (int i = 1; i <= n; ++i) cdf[i] = cdf[i - 1] + tab[i - 1] / (float)n;
    float integral = cdf[n];
    for (int i = 1; i <= n; ++i) cdf[i] = integral == 0.f ? (float)i / (float)n : cdf[i] / integral;
    cdf[n + 1] = sum;
    return tab;
}

/* Triangle::Intersect of an emitter triangle: t and the hit's normal. */
static int emitter_hit(const ctx_t* c, int64_t tr, vec o, vec d, float* t, vec* nn) {
    float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, tt, b1, b2, g[14];
    if (!orc_tri_intersect(c->tris + 9 * tr, oo, dd, 1e-3f, INFINITY, &tt, &b1, &b2)) return 0;
    orc_hit_geometry(c->tris + 9 * tr, c->uvs ? c->uvs + 6 * tr : NULL, oo, dd, tt, b1, b2, g);
    *t = tt;
    *nn = V(g[9], g[10], g[11]);
    return 1;
}

/* A light sample: wi, Li, pdf and the shadow segment's end and eps2;
 * 0 when the sample has no contribution (a parallelogram seen from behind). */
static int sample_light(const ctx_t* c, int l, vec p, float u1, float u2, float comp, vec* wi, vec* Li,
                        float* pdf, vec* target, float* eps2) {
    const orc_light* lt = &c->lights[l];
    if (lt->type == 0) {
        *target = V(lt->pos[0], lt->pos[1], lt->pos[2]);
        *wi = normalize(sub(*target, p));
        *pdf = 1.f;
        vec dv = sub(*target, p);
        float d2 = dot(dv, dv);
        *Li = V(lt->I[0] / d2, lt->I[1] / d2, lt->I[2] / d2);
        *eps2 = 0.f;
        return 1;
    }
    if (lt->type == 2) {
        int n = lt->ntri;
        const float* areas = c->etab[l];
        const float* cdf = areas + n;
        int k = 0;
        while (k < n + 1 && !(cdf[k] > comp)) ++k;
        int sn = k > 0 ? k - 1 : 0;
        const float* v = c->tris + 9 * shape_tri(lt, sn);
        float su1 = sqrtf(u1);
        float b1 = 1.f - su1, b2 = u2 * su1, b0 = 1.f - b1 - b2;
        vec p1 = tri_vertex(v, 0), p2 = tri_vertex(v, 1), p3 = tri_vertex(v, 2);
        vec pt = add(add(scl(p1, b1), scl(p2, b2)), scl(p3, b0));
        vec ns = normalize(cross(sub(p2, p1), sub(p3, p1)));
        vec dir = sub(pt, p);
        float thit = 1.f;
        for (int i = 0; i < n; ++i) {
            float t;
            vec nn;
            if (emitter_hit(c, shape_tri(lt, i), p, dir, &t, &nn)) {
                thit = t;
                ns = nn;
            }
        }
        vec ps = add(p, scl(dir, thit));
        *target = ps;
        *wi = normalize(sub(ps, p));
        float acc = 0.f;
        for (int i = 0; i < n; ++i) {
            float t, pi = 0.f;
            vec nn;
            if (emitter_hit(c, shape_tri(lt, i), p, *wi, &t, &nn)) {
                vec dv = sub(p, add(p, scl(*wi, t)));
                pi = dot(dv, dv) / (fabsf(dot(nn, neg(*wi))) * areas[i]);
                if (isinf(pi)) pi = 0.f;
            }
            acc += areas[i] * pi;
        }
        *pdf = acc / areas[2 * n + 1];
        *Li = dot(ns, neg(*wi)) > 0.f ? V(lt->L[0], lt->L[1], lt->L[2]) : V(0.f, 0.f, 0.f);
        *eps2 = 1e-3f;
        return 1;
    }
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
    *target = add(add(q0, scl(e1, u1)), scl(e3, u2));
    vec dv = sub(*target, p);
    *wi = normalize(dv);
    float d2 = dot(dv, dv);
    float cosl = -dot(n, *wi);
    if (!(cosl > 0.f) || !(d2 > 0.f)) return 0;
    *pdf = d2 / (cosl * area);
    *Li = V(lt->L[0], lt->L[1], lt->L[2]);
    *eps2 = 1e-3f;
    return 1;
}

/* ------------------------------------------------------- the wavefront */

typedef struct {
    vec o, d, beta, L;
    float mint;
    int32_t prim;
    float t, b1, b2;
} path_t;

typedef struct {
    ctx_t* c;
    path_t* P;
    const int64_t* ids;   /* sample index of each slot */
    const int32_t* queue; /* slots to process */
    const int32_t* rank;  /* stream path bounces >= 3: rank among hits */
    int8_t* next;         /* out: the slot continues */
    int64_t begin, end, count, rng_base;
    int bounce;
    uint64_t nearest, shadow;
} stage_t;

static int occluded(stage_t* j, vec o, vec d, float mint, float maxt) {
    float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    j->shadow++;
    return orc_bvh_trace(j->c->bvh, oo, dd, mint, maxt, 1, NULL, NULL, NULL) >= 0;
}

static void* trace_stage(void* arg) {
    stage_t* j = (stage_t*)arg;
    for (int64_t q = j->begin; q < j->end; ++q) {
        path_t* pt = &j->P[j->queue[q]];
        float oo[3] = {pt->o.x, pt->o.y, pt->o.z}, dd[3] = {pt->d.x, pt->d.y, pt->d.z};
        pt->prim = orc_bvh_trace(j->c->bvh, oo, dd, pt->mint, INFINITY, 0, &pt->t, &pt->b1, &pt->b2);
        j->nearest++;
    }
    return NULL;
}

/* One hit of the wavefront: emission, direct lighting, the next direction. */
static void* shade_stage(void* arg) {
    stage_t* j = (stage_t*)arg;
    ctx_t* c = j->c;
    const orc_params* prm = c->prm;
    const int all = prm->integrator == 0;
    const int bounce = j->bounce;
    const int stream = c->s_img != NULL;
    const vec fR = V(prm->albedo[0] * INV_PI, prm->albedo[1] * INV_PI, prm->albedo[2] * INV_PI);
    const int max_depth = prm->max_depth > 0 ? prm->max_depth : 5;
    for (int64_t q = j->begin; q < j->end; ++q) {
        const int32_t slot = j->queue[q];
        path_t* pt = &j->P[slot];
        j->next[q] = 0;
        if (pt->prim < 0) continue;
        const int64_t s = j->ids[slot];
        const float* sd = stream ? c->s_dims + s * c->ndims : NULL;
        float oo[3] = {pt->o.x, pt->o.y, pt->o.z}, dd[3] = {pt->d.x, pt->d.y, pt->d.z}, g[14];
        orc_hit_geometry(c->tris + 9 * (int64_t)pt->prim, c->uvs ? c->uvs + 6 * (int64_t)pt->prim : NULL, oo, dd,
                         pt->t, pt->b1, pt->b2, g);
        vec p = V(g[0], g[1], g[2]), dpdu = V(g[3], g[4], g[5]), nn = V(g[9], g[10], g[11]);
        float eps = 1e-3f * pt->t;
        vec sn = normalize(dpdu), tn = cross(nn, sn);
        vec wo = neg(pt->d);
        vec Le = V(0.f, 0.f, 0.f);
        if (bounce == 0)
            for (int l = 0; l < c->nlights; ++l) {
                const orc_light* lt = &c->lights[l];
                if (lt->type == 2 && pt->prim >= lt->first_tri && pt->prim < lt->first_tri + lt->ntri &&
                    dot(nn, wo) > 0.f)
                    Le = V(lt->L[0], lt->L[1], lt->L[2]);
            }
        float won = dot(wo, nn);
        vec wol = V(dot(wo, sn), dot(wo, tn), dot(wo, nn));
        const float* rv = NULL; /* this ray's UniformSampleOneLight draws (stream path, bounces >= 3) */
        if (stream && !all && bounce >= PATH_SAMPLE_DEPTH) rv = c->s_rng + j->rng_base + 7 * s;
        /* direct lighting */
        vec Ld = V(0.f, 0.f, 0.f);
        int lfirst = 0, llast = c->nlights;
        float pu[3] = {0.f, 0.f, 0.f};
        if (!all && c->nlights > 0) {
            float lnum;
            if (!stream) {
                lnum = rnd(prm->seed, (uint64_t)s, dim_extra(bounce, 15));
                pu[0] = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 0));
                pu[1] = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 1));
                pu[2] = rnd(prm->seed, (uint64_t)s, dim_extra(bounce, 0));
            } else if (bounce < PATH_SAMPLE_DEPTH) {
                lnum = sd[10 * bounce];
                pu[0] = sd[10 * bounce + 1];
                pu[1] = sd[10 * bounce + 2];
                pu[2] = sd[10 * bounce + 3];
            } else {
                lnum = rv[0];
                pu[0] = rv[1];
                pu[1] = rv[2];
                pu[2] = rv[3];
            }
            int ln = (int)floorf(lnum * (float)c->nlights);
            lfirst = ln < c->nlights - 1 ? ln : c->nlights - 1;
            llast = lfirst + 1;
        }
        int m = 0;
        for (int l = lfirst; l < llast; ++l) {
            const orc_light* lt = &c->lights[l];
            int ns = all ? (lt->type == 0 ? 1 : (lt->nsamples > 0 ? lt->nsamples : 1)) : 1;
            for (int qq = 0; qq < ns; ++qq, ++m) {
                float u1, u2, comp;
                if (!all) {
                    u1 = pu[0]; u2 = pu[1]; comp = pu[2];
                } else if (stream) {
                    u1 = sd[6 * m]; u2 = sd[6 * m + 1]; comp = sd[6 * m + 2];
                } else {
                    u1 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 2 * qq));
                    u2 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 2 * qq) + 1);
                    comp = rnd(prm->seed, (uint64_t)s, dim_extra(bounce, m));
                }
                vec wi, Li, target;
                float pdf, eps2;
                if (!sample_light(c, l, p, u1, u2, comp, &wi, &Li, &pdf, &target, &eps2)) continue;
                if (!(pdf > 0.f) || (Li.x == 0.f && Li.y == 0.f && Li.z == 0.f)) continue;
                if (!(dot(wi, nn) * won > 0.f)) continue; /* BSDF::f: reflection only */
                float dist = length(sub(p, target));
                vec dn = scl(sub(target, p), 1.f / dist);
                if (occluded(j, p, dn, eps, dist * (1.f - eps2))) continue;
                float absdot = fabsf(dot(wi, nn));
                vec fL = V(fR.x * Li.x, fR.y * Li.y, fR.z * Li.z);
                vec cc;
                if (lt->type == 0) {
                    if (all) cc = V(fL.x * absdot / pdf, fL.y * absdot / pdf, fL.z * absdot / pdf);
                    else { float w = absdot / pdf; cc = V(fL.x * w, fL.y * w, fL.z * w); }
                } else {
                    vec wil = V(dot(wi, sn), dot(wi, tn), dot(wi, nn));
                    float bpdf = (wol.z * wil.z > 0.f) ? fabsf(wil.z) * INV_PI : 0.f;
                    float f2 = pdf * pdf, g2 = bpdf * bpdf;
                    float weight = f2 / (f2 + g2);
                    if (all)
                        cc = V(fL.x * absdot * weight / pdf, fL.y * absdot * weight / pdf,
                               fL.z * absdot * weight / pdf);
                    else { float w = absdot * weight / pdf; cc = V(fL.x * w, fL.y * w, fL.z * w); }
                }
                if (all) {
                    Ld = add(Ld, cc);
                } else {
                    float fl = (float)c->nlights;
                    Ld = V(cc.x * fl, cc.y * fl, cc.z * fl);
                }
            }
        }
        if (all) {
            pt->L = add(add(pt->L, Ld), Le);
            continue;
        }
        pt->L = add(pt->L, Le);
        pt->L = add(pt->L, V(pt->beta.x * Ld.x, pt->beta.y * Ld.y, pt->beta.z * Ld.z));
        /* cosine-weighted BSDF sample (ConcentricSampleDisk) */
        const float* bv = NULL;
        float u1, u2;
        if (!stream) {
            u1 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 14));
            u2 = rnd(prm->seed, (uint64_t)s, dim_of(bounce, 15));
        } else if (bounce < PATH_SAMPLE_DEPTH) {
            u1 = sd[10 * bounce + 7];
            u2 = sd[10 * bounce + 8];
        } else {
            bv = c->s_rng + j->rng_base + 7 * j->count + (int64_t)j->rank[q] * (bounce > 3 ? 4 : 3);
            u1 = bv[0];
            u2 = bv[1];
        }
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
            float st, ct;
            if (stream) {
                /* theta *= M_PI / 4.f in double, rounded once; sin and cos
                 * correctly rounded (the GPU's choice; the reference takes
                 * the host libm's cosf / sinf) */
                theta = (float)((double)theta * 0.78539816339744830962);
                st = (float)sin((double)theta);
                ct = (float)cos((double)theta);
            } else {
                theta *= 0.785398163397448309616f;
                own_sincos(theta, &st, &ct);
            }
            dx = r * ct;
            dy = r * st;
        }
        vec wil = V(dx, dy, sqrtf(fmaxf(0.f, 1.f - dx * dx - dy * dy)));
        if (wol.z < 0.f) wil.z = -wil.z;
        float pdf = (wol.z * wil.z > 0.f) ? fabsf(wil.z) * INV_PI : 0.f;
        vec wi = V(sn.x * wil.x + tn.x * wil.y + nn.x * wil.z, sn.y * wil.x + tn.y * wil.y + nn.y * wil.z,
                   sn.z * wil.x + tn.z * wil.y + nn.z * wil.z);
        if (!(dot(wi, nn) * won > 0.f) || !(pdf > 0.f)) continue;
        float absdot = fabsf(dot(wi, nn));
        vec beta = V(pt->beta.x * ((fR.x * absdot) / pdf), pt->beta.y * ((fR.y * absdot) / pdf),
                     pt->beta.z * ((fR.z * absdot) / pdf));
        if (bounce > 3) {
            float y = 0.212671f * beta.x + 0.715160f * beta.y + 0.072169f * beta.z;
            float cont = fminf(0.5f, y);
            float u = stream ? bv[3] : rnd(prm->seed, (uint64_t)s, dim_of(bounce, 13));
            if (u > cont) continue;
            beta = V(beta.x / cont, beta.y / cont, beta.z / cont);
        }
        if (bounce == max_depth) continue;
        pt->beta = beta;
        pt->o = p;
        pt->d = wi;
        pt->mint = eps;
        j->next[q] = 1;
    }
    return NULL;
}

static void run_stage(stage_t proto, int64_t nq, int nthreads, void* (*fn)(void*), uint64_t counts[2]) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    stage_t jobs[256];
    pthread_t th[256];
    int64_t chunk = (nq + nthreads - 1) / nthreads;
    int started = 0;
    for (int k = 0; k < nthreads; ++k) {
        jobs[k] = proto;
        jobs[k].begin = k * chunk;
        jobs[k].end = (k + 1) * chunk < nq ? (k + 1) * chunk : nq;
        if (jobs[k].begin >= jobs[k].end) break;
        pthread_create(&th[k], NULL, fn, &jobs[k]);
        started = k + 1;
    }
    for (int k = 0; k < started; ++k) {
        pthread_join(th[k], NULL);
        counts[0] += jobs[k].nearest;
        counts[1] += jobs[k].shadow;
    }
}

/* One task: samples ids[0..m) (stream renders: the stream's positions), as
 * one wavefront; L receives each sample's radiance (indexed by slot). */
static void run_task(ctx_t* c, const int64_t* ids, int64_t m, float* Lout, int nthreads, uint64_t counts[2]) {
    const orc_params* prm = c->prm;
    const orc_camera* cam = c->cam;
    const int spp = prm->spp_x * prm->spp_y;
    path_t* P = (path_t*)malloc(sizeof(path_t) * (size_t)(m > 0 ? m : 1));
    int32_t* queue = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    int32_t* rank = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    int8_t* next = (int8_t*)malloc((size_t)(m > 0 ? m : 1));
    for (int64_t k = 0; k < m; ++k) {
        const int64_t s = ids[k];
        float ix, iy;
        if (c->s_img) {
            ix = c->s_img[2 * s];
            iy = c->s_img[2 * s + 1];
        } else {
            int64_t pix = s / spp;
            int kk = (int)(s % spp);
            int px = (int)(pix % cam->xres), py = (int)(pix / cam->xres);
            int sx = kk % prm->spp_x, sy = kk / prm->spp_x;
            float jx = prm->jitter ? rnd(prm->seed, (uint64_t)s, 0) : 0.5f;
            float jy = prm->jitter ? rnd(prm->seed, (uint64_t)s, 1) : 0.5f;
            ix = ((float)sx + jx) * (1.f / (float)prm->spp_x) + (float)px;
            iy = ((float)sy + jy) * (1.f / (float)prm->spp_y) + (float)py;
        }
        vec pc = xpoint(cam->r2c, V(ix, iy, 0.f));
        P[k].o = xpoint(cam->c2w, V(0.f, 0.f, 0.f));
        P[k].d = xvector(cam->c2w, normalize(pc));
        P[k].mint = 0.f;
        P[k].beta = V(1.f, 1.f, 1.f);
        P[k].L = V(0.f, 0.f, 0.f);
        queue[k] = (int32_t)k;
    }
    int64_t nq = m, rng_base = 0;
    const int stream_draws = c->s_img && prm->integrator == 1;
    for (int bounce = 0; nq > 0; ++bounce) {
        stage_t st;
        memset(&st, 0, sizeof(st));
        st.c = c;
        st.P = P;
        st.ids = ids;
        st.queue = queue;
        st.rank = rank;
        st.next = next;
        st.count = m;
        st.bounce = bounce;
        run_stage(st, nq, nthreads, trace_stage, counts);
        int64_t nhits = 0;
        for (int64_t q = 0; q < nq; ++q) {
            rank[q] = (int32_t)nhits;
            if (P[queue[q]].prim >= 0) ++nhits;
        }
        st.rng_base = rng_base;
        run_stage(st, nq, nthreads, shade_stage, counts);
        if (stream_draws && bounce >= PATH_SAMPLE_DEPTH) rng_base += 7 * m + nhits * (bounce > 3 ? 4 : 3);
        if (prm->integrator != 1) break;
        int64_t w = 0;
        for (int64_t q = 0; q < nq; ++q)
            if (next[q]) queue[w++] = queue[q];
        nq = w;
    }
    for (int64_t k = 0; k < m; ++k) {
        Lout[3 * k] = P[k].L.x;
        Lout[3 * k + 1] = P[k].L.y;
        Lout[3 * k + 2] = P[k].L.z;
    }
    free(P);
    free(queue);
    free(rank);
    free(next);
}

static void ctx_init(ctx_t* c, const float* tris, const float* uvs, void* bvh, const orc_camera* cam,
                     const orc_light* lights, int nlights, const orc_params* prm) {
    memset(c, 0, sizeof(*c));
    c->tris = tris;
    c->uvs = uvs;
    c->bvh = bvh;
    c->cam = cam;
    c->lights = lights;
    c->nlights = nlights < 8 ? nlights : 8;
    c->prm = prm;
    for (int l = 0; l < c->nlights; ++l)
        if (lights[l].type == 2) c->etab[l] = emitter_table(tris, &lights[l]);
}

static void ctx_free(ctx_t* c) {
    for (int l = 0; l < 8; ++l) free(c->etab[l]);
}

/* Radiance -> the film: each sample adds to the pixels of the box filter's
 * footprint (ImageFilm::AddSample), in sample order. */
static void film(const orc_camera* cam, const float* img_xy, const float* L, int64_t n, int spp, float* rgb) {
    const int64_t npix = (int64_t)cam->xres * cam->yres;
    float* acc = (float*)calloc((size_t)npix * 4, sizeof(float));
    for (int64_t s = 0; s < n; ++s) {
        int x0, x1, y0, y1;
        if (img_xy) {
            float dx = img_xy[2 * s] - 0.5f, dy = img_xy[2 * s + 1] - 0.5f;
            x0 = (int)ceilf(dx - 0.5f);
            x1 = (int)floorf(dx + 0.5f);
            y0 = (int)ceilf(dy - 0.5f);
            y1 = (int)floorf(dy + 0.5f);
            if (x0 < 0) x0 = 0;
            if (y0 < 0) y0 = 0;
            if (x1 > cam->xres - 1) x1 = cam->xres - 1;
            if (y1 > cam->yres - 1) y1 = cam->yres - 1;
        } else {
            int64_t pix = s / spp;
            x0 = x1 = (int)(pix % cam->xres);
            y0 = y1 = (int)(pix / cam->xres);
        }
        const float* l = L + 3 * s;
        float r = l[0], g = l[1], b = l[2];
        float lum = 0.212671f * r + 0.715160f * g + 0.072169f * b;
        if (isnan(r) || isnan(g) || isnan(b) || lum < -1e-5f || isinf(lum)) r = g = b = 0.f;
        float x = 0.412453f * r + 0.357580f * g + 0.180423f * b;
        float y = 0.212671f * r + 0.715160f * g + 0.072169f * b;
        float z = 0.019334f * r + 0.119193f * g + 0.950227f * b;
        for (int yy = y0; yy <= y1; ++yy)
            for (int xx = x0; xx <= x1; ++xx) {
                float* a = acc + 4 * ((int64_t)yy * cam->xres + xx);
                a[0] += x;
                a[1] += y;
                a[2] += z;
                a[3] += 1.f;
            }
    }
    for (int64_t p = 0; p < npix; ++p) {
        const float* a = acc + 4 * p;
        float R = 3.240479f * a[0] - 1.537150f * a[1] - 0.498535f * a[2];
        float G = -0.969256f * a[0] + 1.875991f * a[1] + 0.041556f * a[2];
        float B = 0.055648f * a[0] - 0.204043f * a[1] + 1.057311f * a[2];
        if (a[3] != 0.f) {
            float inv = 1.f / a[3];
            R = fmaxf(0.f, R * inv);
            G = fmaxf(0.f, G * inv);
            B = fmaxf(0.f, B * inv);
        }
        rgb[3 * p] = R;
        rgb[3 * p + 1] = G;
        rgb[3 * p + 2] = B;
    }
    free(acc);
}

/* Samples first + k * stride of the frame (k < nslots), task by task. */
static void run_samples(ctx_t* c, float* L, int64_t first, int64_t stride, int64_t nslots, int nthreads,
                        uint64_t counts[2]) {
    int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * TASK_SAMPLES);
    float* Lt = (float*)malloc(sizeof(float) * 3 * TASK_SAMPLES);
    counts[0] = counts[1] = 0;
    for (int64_t k0 = 0; k0 < nslots; k0 += TASK_SAMPLES) {
        int64_t m = nslots - k0 < TASK_SAMPLES ? nslots - k0 : TASK_SAMPLES;
        for (int64_t k = 0; k < m; ++k) ids[k] = first + (k0 + k) * stride;
        run_task(c, ids, m, Lt, nthreads, counts);
        if (L)
            for (int64_t k = 0; k < m; ++k) memcpy(L + 3 * ids[k], Lt + 3 * k, 3 * sizeof(float));
    }
    free(ids);
    free(Lt);
}

/* rgb: [yres][xres][3].  nthreads host threads per wavefront stage. */
void orc_render(const float* tris, int64_t ntri, const orc_camera* cam, const orc_light* lights,
                int nlights, const orc_params* prm, float* rgb, int nthreads) {
    const int spp = prm->spp_x * prm->spp_y;
    const int64_t n = (int64_t)cam->xres * cam->yres * spp;
    float* L = (float*)malloc((size_t)(n > 0 ? n : 1) * 3 * sizeof(float));
    void* bvh = orc_bvh_build(tris, ntri, 4);
    ctx_t c;
    ctx_init(&c, tris, NULL, bvh, cam, lights, nlights, prm);
    uint64_t counts[2];
    run_samples(&c, L, 0, 1, n, nthreads, counts);
    film(cam, NULL, L, n, spp, rgb);
    ctx_free(&c);
    orc_bvh_free(bvh);
    free(L);
}

/* The reference's sample stream: count samples at image_xy, per-sample
 * values dims[count][ndims] and the RNG continuation rng[nrng], in the
 * layout of pbg_sample_stream (include/pbrt_gb300.h).  One task. */
int orc_render_stream(const float* tris, int64_t ntri, const orc_camera* cam, const orc_light* lights,
                      int nlights, const orc_params* prm, int64_t count, const float* image_xy, const float* dims,
                      int ndims, const float* rng, int64_t nrng, float* rgb, int nthreads) {
    if (count <= 0 || count > TASK_SAMPLES) return -1;
    float* L = (float*)malloc((size_t)count * 3 * sizeof(float));
    int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * (size_t)count);
    for (int64_t k = 0; k < count; ++k) ids[k] = k;
    void* bvh = orc_bvh_build(tris, ntri, 4);
    ctx_t c;
    ctx_init(&c, tris, NULL, bvh, cam, lights, nlights, prm);
    c.s_img = image_xy;
    c.s_dims = dims;
    c.ndims = ndims;
    c.s_rng = rng;
    c.nrng = nrng;
    uint64_t counts[2] = {0, 0};
    run_task(&c, ids, count, L, nthreads, counts);
    film(cam, image_xy, L, count, 1, rgb);
    ctx_free(&c);
    orc_bvh_free(bvh);
    free(ids);
    free(L);
    return 0;
}

/* The CPU baseline's bounded sample of a frame: the BVH is built once
 * (orc_render_bvh, degenerate triangles boxed as pbrt's BVHAccel boxes
 * them), then orc_render_count traces the samples first, first + stride,
 * ... of the image and returns only the ray counts. */
void* orc_render_bvh(const float* tris, int64_t ntri) { return orc_bvh_build_mode(tris, ntri, 4, 1); }
void orc_render_bvh_free(void* bvh) { orc_bvh_free(bvh); }
void orc_render_count(const float* tris, void* bvh, const orc_camera* cam, const orc_light* lights,
                      int nlights, const orc_params* prm, int64_t first, int64_t stride, int nthreads,
                      uint64_t* counts) {
    const int64_t n = (int64_t)cam->xres * cam->yres * prm->spp_x * prm->spp_y;
    if (stride < 1) stride = 1;
    const int64_t nslots = first < n ? (n - first + stride - 1) / stride : 0;
    ctx_t c;
    ctx_init(&c, tris, NULL, bvh, cam, lights, nlights, prm);
    run_samples(&c, NULL, first, stride, nslots, nthreads, counts);
    ctx_free(&c);
}

/* The restated DiffuseAreaLight::Sample_L for rows q[n][7] = (p.xyz, eps,
 * u0, u1, comp) over the emitter tris9[ntri]; out rows as the reference
 * harness's ref_area_light_sample: L.rgb, wi.xyz, pdf, the shadow ray's
 * o.xyz, d.xyz, mint, maxt. */
void orc_area_light_sample(const float* tris9, int ntri, const float* L3, const float* q, int64_t n, float* out) {
    orc_light lt;
    memset(&lt, 0, sizeof(lt));
    lt.type = 2;
    lt.nsamples = 1;
    lt.first_tri = 0;
    lt.ntri = ntri;
    lt.L[0] = L3[0]; lt.L[1] = L3[1]; lt.L[2] = L3[2];
    ctx_t c;
    ctx_init(&c, tris9, NULL, NULL, NULL, &lt, 1, NULL);
    for (int64_t i = 0; i < n; ++i) {
        const float* r = q + 7 * i;
        vec p = V(r[0], r[1], r[2]), wi, Li, target;
        float pdf, eps2;
        sample_light(&c, 0, p, r[4], r[5], r[6], &wi, &Li, &pdf, &target, &eps2);
        float dist = length(sub(p, target));
        vec dn = scl(sub(target, p), 1.f / dist);
        float* o = out + 16 * i;
        o[0] = Li.x; o[1] = Li.y; o[2] = Li.z;
        o[3] = wi.x; o[4] = wi.y; o[5] = wi.z;
        o[6] = pdf;
        o[7] = p.x; o[8] = p.y; o[9] = p.z;
        o[10] = dn.x; o[11] = dn.y; o[12] = dn.z;
        o[13] = r[3]; o[14] = dist * (1.f - eps2); o[15] = 0.f;
    }
    ctx_free(&c);
}
