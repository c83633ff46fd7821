/*
 * pbrt_oracle.c -- CPU restatement of the pbrt-v2 ray/triangle path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  The product path (pbrt-v2_gb300/) never links or calls it.
 *
 * What it restates (reference paths are relative to the pbrt-v2 fork's tree):
 *   - Triangle::Intersect / Triangle::IntersectP, shapes/trianglemesh.cpp:119-156
 *     and :203-240, including pbrt's mixed precision: Cross() works in double
 *     (core/geometry.h:481-488) and rounds each component to float, Dot() is
 *     float (core/geometry.h:469-472), invDivisor = 1.f/divisor.
 *   - The differential geometry a hit produces, shapes/trianglemesh.cpp:158-190
 *     (dpdu/dpdv, default uvs from shapes/trianglemesh.h:81-95, the
 *     CoordinateSystem fallback core/geometry.h:512-522) and the surface normal
 *     of DifferentialGeometry's constructor, core/diffgeom.cpp:32-47.
 *   - Aggregate semantics: a sequential loop over primitives in index order
 *     with the ray's maxt shrunk to every accepted hit (the CPU aggregates,
 *     e.g. accelerators/bvh.cpp:464-517), which returns the minimum t and, on
 *     an exact tie in t, the LAST tested (highest index) triangle because the
 *     test rejects only t > maxt.
 *   - A BVH in the style of pbrt's BVHAccel (SAH with 12 buckets, at most 4
 *     primitives per leaf; accelerators/bvh.cpp:209-283, :464-566) used as the
 *     timed CPU baseline.  Its ray/box test is widened so that it never culls a
 *     triangle the exact test accepts, and it applies the same (t, index) rule,
 *     so its answers equal the brute-force loop.
 *
 * Build with -ffp-contract=off: the reference's x86 build has no FMA
 * contraction, and the aarch64 compiler would otherwise fuse a*b+c.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#if defined(__FP_FAST_FMA) && !defined(ORACLE_ALLOW_FMA)
/* nothing: contraction is controlled by -ffp-contract=off on the command line */
#endif

/* ---------------------------------------------------------------- helpers */

/* core/geometry.h:481-488: each component is (v1y*v2z) - (v1z*v2y) in double,
 * rounded to float when the Vector is constructed. */
static inline void cross_pbrt(const float a[3], const float b[3], float out[3]) {
    double ax = a[0], ay = a[1], az = a[2];
    double bx = b[0], by = b[1], bz = b[2];
    out[0] = (float)((ay * bz) - (az * by));
    out[1] = (float)((az * bx) - (ax * bz));
    out[2] = (float)((ax * by) - (ay * bx));
}

/* core/geometry.h:469-472: v1.x*v2.x + v1.y*v2.y + v1.z*v2.z in float. */
static inline float dot_pbrt(const float a[3], const float b[3]) {
    float xx = a[0] * b[0];
    float yy = a[1] * b[1];
    float zz = a[2] * b[2];
    float s = xx + yy;
    return s + zz;
}

/* Ray record used by every oracle entry point: SoA rows of a [8][n] array,
 * rows = ox, oy, oz, dx, dy, dz, mint, maxt. */
typedef struct {
    const float* r;
    int64_t n;
} rays_t;

static inline void ray_get(const float* r, int64_t n, int64_t i, float o[3], float d[3],
                           float* mint, float* maxt) {
    o[0] = r[0 * n + i]; o[1] = r[1 * n + i]; o[2] = r[2 * n + i];
    d[0] = r[3 * n + i]; d[1] = r[4 * n + i]; d[2] = r[5 * n + i];
    *mint = r[6 * n + i]; *maxt = r[7 * n + i];
}

/* ------------------------------------------------- the exact triangle test */

/* shapes/trianglemesh.cpp:119-156 (Intersect) / :203-240 (IntersectP).
 * tri = p1.xyz p2.xyz p3.xyz.  Returns 1 and writes t, b1, b2 on a hit. */
int orc_tri_intersect(const float* tri, const float o[3], const float dir[3], float mint,
                      float maxt, float* t_out, float* b1_out, float* b2_out) {
    const float* p1 = tri;
    const float* p2 = tri + 3;
    const float* p3 = tri + 6;
    float e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    float e2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    float s1[3];
    cross_pbrt(dir, e2, s1);
    float divisor = dot_pbrt(s1, e1);
    if (divisor == 0.)
        return 0;
    float invDivisor = 1.f / divisor;

    float d[3] = {o[0] - p1[0], o[1] - p1[1], o[2] - p1[2]};
    float b1 = dot_pbrt(d, s1) * invDivisor;
    if (b1 < 0. || b1 > 1.)
        return 0;

    float s2[3];
    cross_pbrt(d, e1, s2);
    float b2 = dot_pbrt(dir, s2) * invDivisor;
    if (b2 < 0. || b1 + b2 > 1.)
        return 0;

    float t = dot_pbrt(e2, s2) * invDivisor;
    if (t < mint || t > maxt)
        return 0;
    *t_out = t;
    *b1_out = b1;
    *b2_out = b2;
    return 1;
}

/* ------------------------------------------------------ brute-force loops */

typedef struct {
    const float* tris;
    int64_t ntri;
    const float* rays;
    int64_t n;
    const uint8_t* valid;
    int32_t* prim;
    float* t;
    float* b1;
    float* b2;
    uint8_t* occ;
    int64_t begin, end;
} brute_job_t;

/* Sequential aggregate semantics (accelerators/bvh.cpp:464-517 visits in tree
 * order; here the order is the primitive index): every accepted hit shrinks
 * ray.maxt (core/primitive.cpp GeometricPrimitive::Intersect sets
 * r.maxt = thit), so equal t is accepted again and the last index wins. */
static void* brute_nearest_worker(void* arg) {
    brute_job_t* j = (brute_job_t*)arg;
    for (int64_t i = j->begin; i < j->end; ++i) {
        j->prim[i] = -1;
        j->t[i] = 0.f; j->b1[i] = 0.f; j->b2[i] = 0.f;
        if (j->valid && !j->valid[i]) continue;
        float o[3], d[3], mint, maxt;
        ray_get(j->rays, j->n, i, o, d, &mint, &maxt);
        for (int64_t k = 0; k < j->ntri; ++k) {
            float t, b1, b2;
            if (orc_tri_intersect(j->tris + 9 * k, o, d, mint, maxt, &t, &b1, &b2)) {
                maxt = t;
                j->prim[i] = (int32_t)k;
                j->t[i] = t; j->b1[i] = b1; j->b2[i] = b2;
            }
        }
    }
    return NULL;
}

static void* brute_anyhit_worker(void* arg) {
    brute_job_t* j = (brute_job_t*)arg;
    for (int64_t i = j->begin; i < j->end; ++i) {
        j->occ[i] = 0;
        if (j->valid && !j->valid[i]) continue;
        float o[3], d[3], mint, maxt;
        ray_get(j->rays, j->n, i, o, d, &mint, &maxt);
        for (int64_t k = 0; k < j->ntri; ++k) {
            float t, b1, b2;
            if (orc_tri_intersect(j->tris + 9 * k, o, d, mint, maxt, &t, &b1, &b2)) {
                j->occ[i] = 1;
                break;
            }
        }
    }
    return NULL;
}

static void run_jobs(brute_job_t* proto, void* (*fn)(void*), int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    brute_job_t jobs[256];
    pthread_t th[256];
    int64_t n = proto->n;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    int started = 0;
    for (int k = 0; k < nthreads; ++k) {
        jobs[k] = *proto;
        jobs[k].begin = k * chunk;
        jobs[k].end = (k + 1) * chunk < n ? (k + 1) * chunk : n;
        if (jobs[k].begin >= jobs[k].end) break;
        if (nthreads == 1) { fn(&jobs[k]); started = 0; break; }
        pthread_create(&th[k], NULL, fn, &jobs[k]);
        started = k + 1;
    }
    for (int k = 0; k < started; ++k) pthread_join(th[k], NULL);
}

void orc_nearest_brute(const float* tris, int64_t ntri, const float* rays, int64_t n,
                       const uint8_t* valid, int32_t* prim, float* t, float* b1, float* b2,
                       int nthreads) {
    brute_job_t j = {tris, ntri, rays, n, valid, prim, t, b1, b2, NULL, 0, n};
    run_jobs(&j, brute_nearest_worker, nthreads);
}

void orc_anyhit_brute(const float* tris, int64_t ntri, const float* rays, int64_t n,
                      const uint8_t* valid, uint8_t* occ, int nthreads) {
    brute_job_t j = {tris, ntri, rays, n, valid, NULL, NULL, NULL, NULL, occ, 0, n};
    run_jobs(&j, brute_anyhit_worker, nthreads);
}

/* ---------------------------------------------- differential geometry */

/* shapes/trianglemesh.cpp:158-190 and core/diffgeom.cpp:32-47 for one hit.
 * uv6 = per-triangle (u,v) of its three vertices, or NULL for pbrt's default
 * (0,0),(1,0),(1,1).  out13 = p.xyz dpdu.xyz dpdv.xyz nn.xyz... laid out as
 *   [0..2] p = ray(t) = o + d*t, [3..5] dpdu, [6..8] dpdv, [9..11] nn,
 *   [12] u, [13] v.  (14 floats) */
void orc_hit_geometry(const float* tri, const float* uv6, const float o[3], const float d[3],
                      float t, float b1, float b2, float* out) {
    const float* p1 = tri;
    const float* p2 = tri + 3;
    const float* p3 = tri + 6;
    float uvs[3][2];
    if (uv6) {
        uvs[0][0] = uv6[0]; uvs[0][1] = uv6[1];
        uvs[1][0] = uv6[2]; uvs[1][1] = uv6[3];
        uvs[2][0] = uv6[4]; uvs[2][1] = uv6[5];
    } else {
        uvs[0][0] = 0.f; uvs[0][1] = 0.f;
        uvs[1][0] = 1.f; uvs[1][1] = 0.f;
        uvs[2][0] = 1.f; uvs[2][1] = 1.f;
    }
    float e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    float e2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    float du1 = uvs[0][0] - uvs[2][0];
    float du2 = uvs[1][0] - uvs[2][0];
    float dv1 = uvs[0][1] - uvs[2][1];
    float dv2 = uvs[1][1] - uvs[2][1];
    float dp1[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
    float dp2[3] = {p2[0] - p3[0], p2[1] - p3[1], p2[2] - p3[2]};
    float dpdu[3], dpdv[3];
    float m1 = du1 * dv2;
    float m2 = dv1 * du2;
    float determinant = m1 - m2;
    if (determinant == 0.f) {
        /* CoordinateSystem(Normalize(Cross(e2, e1)), &dpdu, &dpdv) */
        float n[3];
        cross_pbrt(e2, e1, n);
        float len = sqrtf(dot_pbrt(n, n));
        float inv = 1.f / len;
        float v1[3] = {n[0] * inv, n[1] * inv, n[2] * inv};
        if (fabsf(v1[0]) > fabsf(v1[1])) {
            float a = v1[0] * v1[0];
            float c = v1[2] * v1[2];
            float invLen = 1.f / sqrtf(a + c);
            dpdu[0] = -v1[2] * invLen; dpdu[1] = 0.f; dpdu[2] = v1[0] * invLen;
        } else {
            float a = v1[1] * v1[1];
            float c = v1[2] * v1[2];
            float invLen = 1.f / sqrtf(a + c);
            dpdu[0] = 0.f; dpdu[1] = v1[2] * invLen; dpdu[2] = -v1[1] * invLen;
        }
        cross_pbrt(v1, dpdu, dpdv);
    } else {
        float invdet = 1.f / determinant;
        for (int k = 0; k < 3; ++k) {
            float a = dv2 * dp1[k];
            float b = dv1 * dp2[k];
            dpdu[k] = (a - b) * invdet;
            float c = (-du2) * dp1[k];
            float e = du1 * dp2[k];
            dpdv[k] = (c + e) * invdet;
        }
    }
    float b0 = 1 - b1 - b2;
    float tu0 = b0 * uvs[0][0];
    float tu1 = b1 * uvs[1][0];
    float tu2 = b2 * uvs[2][0];
    float tv0 = b0 * uvs[0][1];
    float tv1 = b1 * uvs[1][1];
    float tv2 = b2 * uvs[2][1];
    float tu = (tu0 + tu1) + tu2;
    float tv = (tv0 + tv1) + tv2;
    /* ray(t) = o + d*t (core/geometry.h:322) */
    for (int k = 0; k < 3; ++k) {
        float dt = d[k] * t;
        out[k] = o[k] + dt;
    }
    /* nn = Normalize(Cross(dpdu, dpdv)) (core/diffgeom.cpp:38) */
    float nn[3];
    cross_pbrt(dpdu, dpdv, nn);
    float len = sqrtf(dot_pbrt(nn, nn));
    float inv = 1.f / len;
    for (int k = 0; k < 3; ++k) {
        out[3 + k] = dpdu[k];
        out[6 + k] = dpdv[k];
        out[9 + k] = nn[k] * inv;
    }
    out[12] = tu;
    out[13] = tv;
    (void)e1;
}

/* Batch form: geometry for every ray with prim >= 0; rows of out are zero
 * for misses.  out is [n][14]. */
void orc_hits_geometry(const float* tris, const float* uvs, const float* rays, int64_t n,
                       const int32_t* prim, const float* t, const float* b1, const float* b2,
                       float* out) {
    for (int64_t i = 0; i < n; ++i) {
        float* row = out + 14 * i;
        if (prim[i] < 0) { memset(row, 0, 14 * sizeof(float)); continue; }
        float o[3], d[3], mint, maxt;
        ray_get(rays, n, i, o, d, &mint, &maxt);
        orc_hit_geometry(tris + 9 * (int64_t)prim[i], uvs ? uvs + 6 * (int64_t)prim[i] : NULL, o,
                         d, t[i], b1[i], b2[i], row);
    }
}

/* --------------------------------------------------------- BVH baseline */

/* Node layout of the flattened tree (accelerators/bvh.cpp LinearBVHNode): a
 * box, and either (first primitive, count) for a leaf or the second child's
 * offset; the first child follows its parent. */
typedef struct {
    float lo[3], hi[3];
    int32_t offset; /* leaf: first primitive in order[]; inner: second child */
    int32_t count;  /* >0 leaf */
    int32_t axis;
} bvh_node_t;

typedef struct {
    bvh_node_t* nodes;
    int64_t nnodes, cap;
    int32_t* order; /* primitive indices in leaf order */
    const float* tris;
    int64_t ntri;
    int32_t* unculled; /* degenerate triangles, tested by every ray */
    int64_t nunculled;
} bvh_t;

/* A triangle whose area is negligible against its edge lengths (or that has
 * a non-finite vertex) is accepted by pbrt's test at points unrelated to its
 * box (the divisor is rounding noise), so no box may cull it: such triangles
 * are kept out of the tree and tested by every ray. */
int orc_tri_degenerate(const float* v) {
    double e1[3], e2[3], c[3];
    for (int k = 0; k < 9; ++k)
        if (!isfinite(v[k])) return 1;
    for (int k = 0; k < 3; ++k) { e1[k] = (double)v[3 + k] - v[k]; e2[k] = (double)v[6 + k] - v[k]; }
    c[0] = e1[1] * e2[2] - e1[2] * e2[1];
    c[1] = e1[2] * e2[0] - e1[0] * e2[2];
    c[2] = e1[0] * e2[1] - e1[1] * e2[0];
    double a2 = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    double l1 = (fabs(e1[0]) + fabs(e1[1]) + fabs(e1[2])) * (fabs(e2[0]) + fabs(e2[1]) + fabs(e2[2]));
    return !(a2 > 0x1p-16 * l1);
}

typedef struct {
    float lo[3], hi[3], c[3];
} prim_info_t;

static int64_t bvh_push(bvh_t* b) {
    if (b->nnodes == b->cap) {
        b->cap = b->cap ? b->cap * 2 : 1024;
        b->nodes = (bvh_node_t*)realloc(b->nodes, b->cap * sizeof(bvh_node_t));
    }
    return b->nnodes++;
}

static float box_area(const float lo[3], const float hi[3]) {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0.f;
    return 2.f * (dx * dy + dx * dz + dy * dz);
}

static int cmp_axis;
static const prim_info_t* cmp_info;
static int cmp_centroid(const void* a, const void* b) {
    float ca = cmp_info[*(const int32_t*)a].c[cmp_axis];
    float cb = cmp_info[*(const int32_t*)b].c[cmp_axis];
    return (ca < cb) ? -1 : (ca > cb) ? 1 : 0;
}

/* SAH recursive build in the manner of accelerators/bvh.cpp:290-420: 12
 * buckets over the centroid extent, cost 1/8 per traversal step, leaf when
 * the split does not pay and the node holds at most maxprims primitives. */
static int64_t bvh_build_rec(bvh_t* b, const prim_info_t* info, int32_t* idx, int64_t start,
                             int64_t end, int maxprims) {
    int64_t node = bvh_push(b);
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = start; i < end; ++i) {
        const prim_info_t* p = &info[idx[i]];
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], p->lo[k]); hi[k] = fmaxf(hi[k], p->hi[k]);
            clo[k] = fminf(clo[k], p->c[k]); chi[k] = fmaxf(chi[k], p->c[k]);
        }
    }
    int64_t np = end - start;
    int axis = 0;
    float ext = chi[0] - clo[0];
    if (chi[1] - clo[1] > ext) { axis = 1; ext = chi[1] - clo[1]; }
    if (chi[2] - clo[2] > ext) { axis = 2; ext = chi[2] - clo[2]; }
    int leaf = (np == 1) || !(ext > 0.f);
    int64_t mid = start + np / 2;
    if (!leaf) {
        if (np <= 4) {
            cmp_axis = axis; cmp_info = info;
            qsort(idx + start, (size_t)np, sizeof(int32_t), cmp_centroid);
            mid = start + np / 2;
        } else {
            enum { NB = 12 };
            int count[NB] = {0};
            float blo[NB][3], bhi[NB][3];
            for (int k = 0; k < NB; ++k)
                for (int a = 0; a < 3; ++a) { blo[k][a] = INFINITY; bhi[k][a] = -INFINITY; }
            for (int64_t i = start; i < end; ++i) {
                const prim_info_t* p = &info[idx[i]];
                int bk = (int)(NB * ((p->c[axis] - clo[axis]) / ext));
                if (bk >= NB) bk = NB - 1;
                if (bk < 0) bk = 0;
                count[bk]++;
                for (int a = 0; a < 3; ++a) {
                    blo[bk][a] = fminf(blo[bk][a], p->lo[a]);
                    bhi[bk][a] = fmaxf(bhi[bk][a], p->hi[a]);
                }
            }
            float cost[NB - 1];
            float area = box_area(lo, hi);
            for (int s = 0; s < NB - 1; ++s) {
                float l0[3] = {INFINITY, INFINITY, INFINITY}, h0[3] = {-INFINITY, -INFINITY, -INFINITY};
                float l1[3] = {INFINITY, INFINITY, INFINITY}, h1[3] = {-INFINITY, -INFINITY, -INFINITY};
                int c0 = 0, c1 = 0;
                for (int k = 0; k <= s; ++k) {
                    c0 += count[k];
                    for (int a = 0; a < 3; ++a) { l0[a] = fminf(l0[a], blo[k][a]); h0[a] = fmaxf(h0[a], bhi[k][a]); }
                }
                for (int k = s + 1; k < NB; ++k) {
                    c1 += count[k];
                    for (int a = 0; a < 3; ++a) { l1[a] = fminf(l1[a], blo[k][a]); h1[a] = fmaxf(h1[a], bhi[k][a]); }
                }
                cost[s] = .125f + (c0 * box_area(l0, h0) + c1 * box_area(l1, h1)) / (area > 0 ? area : 1.f);
            }
            int best = 0;
            for (int s = 1; s < NB - 1; ++s) if (cost[s] < cost[best]) best = s;
            if (np > maxprims || cost[best] < (float)np) {
                /* partition by bucket */
                int64_t i = start, j = end - 1;
                while (i <= j) {
                    const prim_info_t* p = &info[idx[i]];
                    int bk = (int)(NB * ((p->c[axis] - clo[axis]) / ext));
                    if (bk >= NB) bk = NB - 1;
                    if (bk < 0) bk = 0;
                    if (bk <= best) ++i;
                    else { int32_t tmp = idx[i]; idx[i] = idx[j]; idx[j] = tmp; --j; }
                }
                mid = i;
                if (mid == start || mid == end) mid = start + np / 2;
            } else {
                leaf = 1;
            }
        }
    }
    bvh_node_t* nd = &b->nodes[node];
    for (int k = 0; k < 3; ++k) { nd->lo[k] = lo[k]; nd->hi[k] = hi[k]; }
    nd->axis = axis;
    if (leaf) {
        nd->offset = (int32_t)start;
        nd->count = (int32_t)np;
        return node;
    }
    nd->count = 0;
    bvh_build_rec(b, info, idx, start, mid, maxprims);
    int64_t second = bvh_build_rec(b, info, idx, mid, end, maxprims);
    b->nodes[node].offset = (int32_t)second;
    return node;
}

/* box_degenerate = 0: degenerate triangles stay out of the tree and every
 * ray tests them (answers equal the all-pairs loop).  1: they go into the
 * tree with their own boxes, as pbrt's BVHAccel puts every primitive
 * (accelerators/bvh.cpp:220-229); a rounding-noise hit of such a triangle
 * far from its box is then missed, as BVHAccel misses it.  The timed CPU
 * samples use 1, the parity checks 0. */
void* orc_bvh_build_mode(const float* tris, int64_t ntri, int maxprims, int box_degenerate);

void* orc_bvh_build(const float* tris, int64_t ntri, int maxprims) {
    return orc_bvh_build_mode(tris, ntri, maxprims, 0);
}

void* orc_bvh_build_mode(const float* tris, int64_t ntri, int maxprims, int box_degenerate) {
    bvh_t* b = (bvh_t*)calloc(1, sizeof(bvh_t));
    b->tris = tris;
    b->ntri = ntri;
    b->order = (int32_t*)malloc((ntri > 0 ? ntri : 1) * sizeof(int32_t));
    prim_info_t* info = (prim_info_t*)malloc((ntri > 0 ? ntri : 1) * sizeof(prim_info_t));
    b->unculled = (int32_t*)malloc((ntri > 0 ? ntri : 1) * sizeof(int32_t));
    int64_t ncull = 0;
    for (int64_t i = 0; i < ntri; ++i) {
        const float* v = tris + 9 * i;
        int finite = 1;
        for (int k = 0; k < 9; ++k) finite &= isfinite(v[k]) ? 1 : 0;
        /* a non-finite vertex has no box: always tested */
        if ((!box_degenerate || !finite) && orc_tri_degenerate(v)) {
            b->unculled[b->nunculled++] = (int32_t)i;
            continue;
        }
        for (int k = 0; k < 3; ++k) {
            float a = v[k], c = v[3 + k], e = v[6 + k];
            info[ncull].lo[k] = fminf(a, fminf(c, e));
            info[ncull].hi[k] = fmaxf(a, fmaxf(c, e));
            info[ncull].c[k] = .5f * info[ncull].lo[k] + .5f * info[ncull].hi[k];
        }
        b->order[ncull] = (int32_t)i;
        ++ncull;
    }
    /* info[] is indexed by position in order[]; remap so the build sorts order. */
    int32_t* pos = (int32_t*)malloc((ncull > 0 ? ncull : 1) * sizeof(int32_t));
    prim_info_t* info2 = (prim_info_t*)malloc((ncull > 0 ? ncull : 1) * sizeof(prim_info_t));
    for (int64_t i = 0; i < ncull; ++i) { pos[i] = (int32_t)i; info2[i] = info[i]; }
    if (ncull > 0) bvh_build_rec(b, info2, pos, 0, ncull, maxprims);
    for (int64_t i = 0; i < ncull; ++i) pos[i] = b->order[pos[i]];
    memcpy(b->order, pos, (ncull > 0 ? ncull : 1) * sizeof(int32_t));
    free(pos);
    free(info2);
    free(info);
    /* the traversal tests the padded boxes: pad each node once here */
    for (int64_t k = 0; k < b->nnodes; ++k) {
        bvh_node_t* nd = &b->nodes[k];
        for (int a = 0; a < 3; ++a) {
            float pad = (fabsf(nd->lo[a]) + fabsf(nd->hi[a]) + (nd->hi[a] - nd->lo[a])) * 0x1p-10f + 1e-30f;
            float lo = nd->lo[a] - pad, hi = nd->hi[a] + pad;
            nd->lo[a] = lo;
            nd->hi[a] = hi;
        }
    }
    return b;
}

void orc_bvh_free(void* p) {
    bvh_t* b = (bvh_t*)p;
    if (!b) return;
    free(b->nodes);
    free(b->order);
    free(b->unculled);
    free(b);
}

int64_t orc_bvh_node_count(void* p) { return ((bvh_t*)p)->nnodes; }

/* Slab test (accelerators/bvh.cpp:430-460 form) on a box padded by a relative
 * 2^-10 of its extent and magnitude (done once, after the build), with the far
 * distance widened by 2^-10, so that float rounding never culls a triangle
 * that the exact test accepts. */
static inline int box_hit(const bvh_node_t* nd, const float o[3], const float inv[3],
                          const int dirneg[3], float mint, float maxt) {
    float t0 = mint, t1 = maxt;
    for (int a = 0; a < 3; ++a) {
        const float lo = nd->lo[a], hi = nd->hi[a];
        /* near and far planes by the direction's sign (a padded box has
         * lo < hi, so this equals ordering the two distances) */
        float tn = ((dirneg[a] ? hi : lo) - o[a]) * inv[a];
        float tf = ((dirneg[a] ? lo : hi) - o[a]) * inv[a];
        tf *= 1.f + 0x1p-10f;
        if (!(tn <= tf)) { /* NaN from 0*inf: the ray lies in the slab plane */
            if (o[a] >= lo && o[a] <= hi) continue;
            return 0;
        }
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return 0;
    }
    return 1;
}

typedef struct {
    bvh_t* b;
    const float* rays;
    int64_t n;
    const uint8_t* valid;
    int32_t* prim;
    float *t, *b1, *b2;
    uint8_t* occ;
    int64_t begin, end;
} bvh_job_t;

static void bvh_trace_one(bvh_t* b, const float o[3], const float d[3], float mint, float maxt,
                          int anyhit, int32_t* prim, float* tout, float* b1o, float* b2o) {
    float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
    int dirneg[3] = {inv[0] < 0, inv[1] < 0, inv[2] < 0};
    int32_t stack[128];
    int sp = 0;
    int64_t node = 0;
    int32_t best = -1;
    float bt = 0.f, bb1 = 0.f, bb2 = 0.f;
    float curmax = maxt;
    for (int64_t k = 0; k < b->nunculled; ++k) {
        int32_t tri = b->unculled[k];
        float t, u1, u2;
        if (orc_tri_intersect(b->tris + 9 * (int64_t)tri, o, d, mint, curmax, &t, &u1, &u2)) {
            if (best < 0 || t < bt || tri > best) {
                best = tri; bt = t; bb1 = u1; bb2 = u2; curmax = t;
                if (anyhit) { *prim = best; return; }
            }
        }
    }
    if (b->nnodes == 0) {
        *prim = best;
        if (best >= 0) { *tout = bt; *b1o = bb1; *b2o = bb2; }
        return;
    }
    while (1) {
        const bvh_node_t* nd = &b->nodes[node];
        if (box_hit(nd, o, inv, dirneg, mint, curmax)) {
            if (nd->count > 0) {
                for (int32_t k = 0; k < nd->count; ++k) {
                    int32_t tri = b->order[nd->offset + k];
                    float t, u1, u2;
                    if (orc_tri_intersect(b->tris + 9 * (int64_t)tri, o, d, mint, curmax, &t, &u1, &u2)) {
                        if (best < 0 || t < bt || tri > best) {
                            best = tri; bt = t; bb1 = u1; bb2 = u2; curmax = t;
                            if (anyhit) { *prim = best; return; }
                        }
                    }
                }
                if (sp == 0) break;
                node = stack[--sp];
            } else {
                if (dirneg[nd->axis]) { stack[sp++] = (int32_t)(node + 1); node = nd->offset; }
                else { stack[sp++] = nd->offset; node = node + 1; }
            }
        } else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    *prim = best;
    if (best >= 0) { *tout = bt; *b1o = bb1; *b2o = bb2; }
}

/* One ray through the BVH baseline; returns the hit index or -1. */
int32_t orc_bvh_trace(void* bvh, const float o[3], const float d[3], float mint, float maxt,
                      int anyhit, float* t, float* b1, float* b2) {
    int32_t prim = -1;
    float tt = 0.f, u1 = 0.f, u2 = 0.f;
    bvh_trace_one((bvh_t*)bvh, o, d, mint, maxt, anyhit, &prim, &tt, &u1, &u2);
    if (t) *t = tt;
    if (b1) *b1 = u1;
    if (b2) *b2 = u2;
    return prim;
}

static void* bvh_nearest_worker(void* arg) {
    bvh_job_t* j = (bvh_job_t*)arg;
    for (int64_t i = j->begin; i < j->end; ++i) {
        j->prim[i] = -1; j->t[i] = 0.f; j->b1[i] = 0.f; j->b2[i] = 0.f;
        if (j->valid && !j->valid[i]) continue;
        float o[3], d[3], mint, maxt;
        ray_get(j->rays, j->n, i, o, d, &mint, &maxt);
        bvh_trace_one(j->b, o, d, mint, maxt, 0, &j->prim[i], &j->t[i], &j->b1[i], &j->b2[i]);
    }
    return NULL;
}

static void* bvh_anyhit_worker(void* arg) {
    bvh_job_t* j = (bvh_job_t*)arg;
    for (int64_t i = j->begin; i < j->end; ++i) {
        j->occ[i] = 0;
        if (j->valid && !j->valid[i]) continue;
        float o[3], d[3], mint, maxt, t, u1, u2;
        int32_t p = -1;
        ray_get(j->rays, j->n, i, o, d, &mint, &maxt);
        bvh_trace_one(j->b, o, d, mint, maxt, 1, &p, &t, &u1, &u2);
        j->occ[i] = p >= 0;
    }
    return NULL;
}

static void run_bvh_jobs(bvh_job_t* proto, void* (*fn)(void*), int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    bvh_job_t jobs[256];
    pthread_t th[256];
    int64_t n = proto->n;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    int started = 0;
    for (int k = 0; k < nthreads; ++k) {
        jobs[k] = *proto;
        jobs[k].begin = k * chunk;
        jobs[k].end = (k + 1) * chunk < n ? (k + 1) * chunk : n;
        if (jobs[k].begin >= jobs[k].end) break;
        if (nthreads == 1) { fn(&jobs[k]); break; }
        pthread_create(&th[k], NULL, fn, &jobs[k]);
        started = k + 1;
    }
    for (int k = 0; k < started; ++k) pthread_join(th[k], NULL);
}

void orc_bvh_nearest(void* bvh, const float* rays, int64_t n, const uint8_t* valid, int32_t* prim,
                     float* t, float* b1, float* b2, int nthreads) {
    bvh_job_t j = {(bvh_t*)bvh, rays, n, valid, prim, t, b1, b2, NULL, 0, n};
    run_bvh_jobs(&j, bvh_nearest_worker, nthreads);
}

void orc_bvh_anyhit(void* bvh, const float* rays, int64_t n, const uint8_t* valid, uint8_t* occ,
                    int nthreads) {
    bvh_job_t j = {(bvh_t*)bvh, rays, n, valid, NULL, NULL, NULL, NULL, occ, 0, n};
    run_bvh_jobs(&j, bvh_anyhit_worker, nthreads);
}
