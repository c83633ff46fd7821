// ref_harness.cpp -- C entry points into the reference's own CPU classes.
//
// TEST INFRASTRUCTURE ONLY.  Compiled against the unmodified pbrt-v2 fork
// sources (shapes/trianglemesh.cpp, accelerators/bvh.cpp and the core files
// they need) by oracle/ref/Makefile into oracle/_ref/libpbrtref.so.  It is used
// to pin the C restatement in oracle/pbrt_oracle.c and to generate the golden
// fixtures under tests/golden/; nothing on the GPU side loads it.
//
// Every answer comes from pbrt's own code:
//   - Triangle::Intersect / IntersectP   shapes/trianglemesh.cpp:119-245
//   - GeometricPrimitive::Intersect      core/primitive.cpp:88-100 (maxt update)
//   - BVHAccel::Intersect / IntersectP   accelerators/bvh.cpp:464-566
//   - DifferentialGeometry               core/diffgeom.cpp:32-47
// The triangle index of a hit is recovered from Intersection::primitiveId
// (core/intersection.h:52), which counts GeometricPrimitive construction order.
// Barycentrics are recovered exactly by giving every triangle the vertex
// uvs (0,0), (1,0), (0,1): pbrt's interpolation b0*u0 + b1*u1 + b2*u2 then
// returns u = b1 and v = b2 bit for bit.
#include "stdafx.h"
#include "pbrt.h"
#include "primitive.h"
#include "intersection.h"
#include "shapes/trianglemesh.h"
#include "accelerators/bvh.h"
#include "transform.h"
#include "texture.h"
#include "material.h"

#include <stdint.h>
#include <vector>

// Globals that pbrt's api.cpp and parser would define; the harness links
// neither (core/pbrt.h:126, core/error.cpp:62-67).
Options PbrtOptions;
string current_file;
int line_num = 0;

struct RefScene {
    Transform* identity;
    Reference<TriangleMesh> mesh;
    vector<Reference<Primitive> > prims;
    BVHAccel* bvh;
    uint32_t firstId;
    int64_t ntri;
};

extern "C" {

// uv_mode: 0 = no uvs (pbrt's defaults), 1 = barycentric probe uvs,
// 2 = caller uvs (uv6 = 6 floats per triangle).
void* ref_scene_create(const float* tris9, int64_t ntri, int uv_mode, const float* uv6,
                       int bvh_maxprims) {
    RefScene* s = new RefScene();
    s->identity = new Transform();
    s->ntri = ntri;
    int nv = (int)(3 * ntri);
    std::vector<int> vi(nv);
    std::vector<Point> P(nv);
    std::vector<float> uv;
    for (int i = 0; i < nv; ++i) {
        vi[i] = i;
        P[i] = Point(tris9[3 * i], tris9[3 * i + 1], tris9[3 * i + 2]);
    }
    if (uv_mode == 1) {
        uv.resize(2 * nv);
        for (int64_t k = 0; k < ntri; ++k) {
            float* u = &uv[6 * k];
            u[0] = 0.f; u[1] = 0.f; u[2] = 1.f; u[3] = 0.f; u[4] = 0.f; u[5] = 1.f;
        }
    } else if (uv_mode == 2) {
        uv.assign(uv6, uv6 + 6 * ntri);
    }
    s->mesh = new TriangleMesh(s->identity, s->identity, false, (int)ntri, nv,
                               vi.empty() ? NULL : &vi[0], P.empty() ? NULL : &P[0], NULL, NULL,
                               uv.empty() ? NULL : &uv[0], Reference<Texture<float> >(NULL));
    vector<Reference<Shape> > tris;
    s->mesh->Refine(tris);
    s->firstId = 0;
    for (size_t i = 0; i < tris.size(); ++i) {
        GeometricPrimitive* gp =
            new GeometricPrimitive(tris[i], Reference<Material>(NULL), NULL);
        if (i == 0) s->firstId = gp->primitiveId;
        s->prims.push_back(gp);
    }
    s->bvh = bvh_maxprims > 0 ? new BVHAccel(s->prims, (uint32_t)bvh_maxprims, "sah") : NULL;
    return s;
}

void ref_scene_destroy(void* p) {
    RefScene* s = (RefScene*)p;
    if (!s) return;
    delete s->bvh;
    s->prims.clear();
    s->mesh = NULL;
    delete s->identity;
    delete s;
}

static Ray make_ray(const float* rays, int64_t n, int64_t i) {
    Point o(rays[0 * n + i], rays[1 * n + i], rays[2 * n + i]);
    Vector d(rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]);
    return Ray(o, d, rays[6 * n + i], rays[7 * n + i]);
}

// Nearest hit for every ray.  use_bvh = 0: the primitives in index order
// with pbrt's maxt update (the semantics of a sequential aggregate);
// use_bvh = 1: pbrt's BVHAccel.  geo (optional, [n][14]) receives
// p, dpdu, dpdv, nn, u, v of the hit's DifferentialGeometry.
void ref_nearest(void* p, const float* rays, int64_t n, int use_bvh, int32_t* prim, float* t,
                 float* u, float* v, float* geo) {
    RefScene* s = (RefScene*)p;
    for (int64_t i = 0; i < n; ++i) {
        Ray r = make_ray(rays, n, i);
        Intersection isect;
        bool hit = false;
        if (use_bvh) {
            hit = s->bvh->Intersect(r, &isect);
        } else {
            for (size_t k = 0; k < s->prims.size(); ++k)
                if (s->prims[k]->Intersect(r, &isect)) hit = true;
        }
        if (hit) {
            prim[i] = (int32_t)(isect.primitiveId - s->firstId);
            t[i] = r.maxt;
            u[i] = isect.dg.u;
            v[i] = isect.dg.v;
            if (geo) {
                float* g = geo + 14 * i;
                const DifferentialGeometry& dg = isect.dg;
                g[0] = dg.p.x; g[1] = dg.p.y; g[2] = dg.p.z;
                g[3] = dg.dpdu.x; g[4] = dg.dpdu.y; g[5] = dg.dpdu.z;
                g[6] = dg.dpdv.x; g[7] = dg.dpdv.y; g[8] = dg.dpdv.z;
                g[9] = dg.nn.x; g[10] = dg.nn.y; g[11] = dg.nn.z;
                g[12] = dg.u; g[13] = dg.v;
            }
        } else {
            prim[i] = -1;
            t[i] = 0.f; u[i] = 0.f; v[i] = 0.f;
            if (geo)
                for (int k = 0; k < 14; ++k) geo[14 * i + k] = 0.f;
        }
    }
}

// Shadow any-hit for every ray: 1 if some triangle is hit in [mint, maxt].
void ref_anyhit(void* p, const float* rays, int64_t n, int use_bvh, uint8_t* occ) {
    RefScene* s = (RefScene*)p;
    for (int64_t i = 0; i < n; ++i) {
        Ray r = make_ray(rays, n, i);
        bool hit = false;
        if (use_bvh) {
            hit = s->bvh->IntersectP(r);
        } else {
            for (size_t k = 0; k < s->prims.size() && !hit; ++k)
                hit = s->prims[k]->IntersectP(r);
        }
        occ[i] = hit ? 1 : 0;
    }
}

}  // extern "C"

// ------------------------------------------------------------ camera
#include "cameras/perspective.h"
#include "film.h"
#include "camera.h"
#include "sampler.h"

namespace {
// A film that only carries the resolution the camera reads.
struct SizeFilm : public Film {
    SizeFilm(int x, int y) : Film(x, y) {}
    void AddSample(const CameraSample&, const Spectrum&) {}
    void Splat(const CameraSample&, const Spectrum&) {}
    void GetSampleExtent(int* a, int* b, int* c, int* d) const { *a = 0; *b = xResolution; *c = 0; *d = yResolution; }
    void GetPixelExtent(int* a, int* b, int* c, int* d) const { *a = 0; *b = xResolution; *c = 0; *d = yResolution; }
    void WriteImage(float) {}
};
// Exposes ProjectiveCamera's protected RasterToCamera.
struct ExposedCamera : public PerspectiveCamera {
    ExposedCamera(const AnimatedTransform& c2w, const float sw[4], float fov, Film* f)
        : PerspectiveCamera(c2w, sw, 0.f, 1.f, 0.f, 1e30f, fov, f) {}
    const Transform& r2c() const { return RasterToCamera; }
};
}  // namespace

extern "C" {

// pbrt's PerspectiveCamera for LookAt(eye, look, up) + Camera "perspective"
// "fov", the way the scene-file API builds it (core/api.cpp pbrtLookAt,
// MakeCamera; cameras/perspective.cpp CreatePerspectiveCamera with the
// default screen window).  Writes RasterToCamera and CameraToWorld
// (row-major) and the GenerateRayDifferential ray (o, d) of each raster
// sample (xy[2*i], xy[2*i+1]) into rays6[6*i].
void ref_camera(int xres, int yres, const float* eye, const float* look, const float* up, float fov,
                float* r2c16, float* c2w16, const float* xy, int64_t n, float* rays6) {
    Transform w2c = LookAt(Point(eye[0], eye[1], eye[2]), Point(look[0], look[1], look[2]),
                           Vector(up[0], up[1], up[2]));
    Transform c2w = Inverse(w2c);
    AnimatedTransform at(&c2w, 0.f, &c2w, 1.f);
    float frame = float(xres) / float(yres);
    float sw[4];
    if (frame > 1.f) { sw[0] = -frame; sw[1] = frame; sw[2] = -1.f; sw[3] = 1.f; }
    else { sw[0] = -1.f; sw[1] = 1.f; sw[2] = -1.f / frame; sw[3] = 1.f / frame; }
    // Camera's destructor deletes its film (core/camera.cpp), so it is heap-allocated.
    ExposedCamera cam(at, sw, fov, new SizeFilm(xres, yres));
    const Matrix4x4& a = cam.r2c().GetMatrix();
    const Matrix4x4& b = c2w.GetMatrix();
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            r2c16[4 * i + j] = a.m[i][j];
            c2w16[4 * i + j] = b.m[i][j];
        }
    for (int64_t i = 0; i < n; ++i) {
        CameraSample s;
        s.imageX = xy[2 * i];
        s.imageY = xy[2 * i + 1];
        s.lensU = s.lensV = 0.5f;
        s.time = 0.f;
        RayDifferential r;
        cam.GenerateRayDifferential(s, &r);
        float* o = rays6 + 6 * i;
        o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z;
        o[3] = r.d.x; o[4] = r.d.y; o[5] = r.d.z;
    }
}

}  // extern "C"

// ------------------------------------------------------------------ samples
// One breadth-first task's samples from pbrt's own StratifiedSampler and RNG
// (renderers/breadth-first.cpp:18-48, samplers/stratified.cpp:60-105), in
// the layout of orc_pbrt_task_samples (oracle/pbrt_sampler.c), which it pins.
#include "sampler.h"
#include "samplers/stratified.h"
#include "rng.h"

extern "C" {

int64_t ref_task_samples(uint32_t task, int x0, int x1, int y0, int y1, int spx, int spy, int jitter,
                         const int* n1d, int k1, const int* n2d, int k2, int64_t count, float* image_xy,
                         float* oned, float* twod, int64_t nrng, float* rng_out) {
    StratifiedSampler sampler(x0, x1, y0, y1, spx, spy, jitter != 0, 0.f, 1.f);
    Sample proto(NULL, NULL, NULL, NULL);
    for (int k = 0; k < k1; ++k) proto.Add1D(n1d[k]);
    for (int k = 0; k < k2; ++k) proto.Add2D(n2d[k]);
    Sample* samples = proto.Duplicate((int)count);
    RNG rng(task);
    int64_t got = 0;
    while (got < count) {
        int n = sampler.GetMoreSamples(&samples[got], rng);
        if (n == 0) break;
        got += n;
    }
    int t1 = 0, t2 = 0;
    for (int k = 0; k < k1; ++k) t1 += n1d[k];
    for (int k = 0; k < k2; ++k) t2 += n2d[k];
    for (int64_t i = 0; i < got; ++i) {
        image_xy[2 * i] = samples[i].imageX;
        image_xy[2 * i + 1] = samples[i].imageY;
        float* o1 = oned + i * t1;
        for (int k = 0; k < k1; ++k)
            for (int j = 0; j < n1d[k]; ++j) *o1++ = samples[i].oneD[k][j];
        float* o2 = twod + i * 2 * t2;
        for (int k = 0; k < k2; ++k)
            for (int j = 0; j < 2 * n2d[k]; ++j) *o2++ = samples[i].twoD[k][j];
    }
    for (int64_t k = 0; k < nrng; ++k) rng_out[k] = rng.RandomFloat();
    delete[] samples;
    return got;
}

}  // extern "C"

// ------------------------------------------------------------- area light
// pbrt's DiffuseAreaLight over a triangle mesh (lights/diffuse.cpp:61-79):
// for each (p, eps, uPos[0], uPos[1], uComponent) row, Sample_L's radiance,
// wi, pdf and shadow segment.  Pins the restatement of the light sampling.
#include "lights/diffuse.h"

extern "C" {

// tris9: the emitter's triangles; q[n][5] = p.xyz... no: q rows are
// (px, py, pz, eps, u0, u1, comp); out rows: L.rgb, wi.xyz, pdf, ray o.xyz,
// d.xyz, mint, maxt (16 floats).
void ref_area_light_sample(const float* tris9, int ntri, const float* L3, const float* q, int64_t n,
                           float* out) {
    Transform* identity = new Transform();
    int nv = 3 * ntri;
    std::vector<int> vi(nv);
    std::vector<Point> P(nv);
    for (int i = 0; i < nv; ++i) {
        vi[i] = i;
        P[i] = Point(tris9[3 * i], tris9[3 * i + 1], tris9[3 * i + 2]);
    }
    Reference<Shape> mesh = new TriangleMesh(identity, identity, false, ntri, nv, &vi[0], &P[0], NULL, NULL,
                                             NULL, NULL);
    float rgb[3] = {L3[0], L3[1], L3[2]};
    DiffuseAreaLight light(Transform(), RGBSpectrum::FromRGB(rgb), 1, mesh);
    for (int64_t i = 0; i < n; ++i) {
        const float* r = q + 7 * i;
        LightSample ls(r[4], r[5], r[6]);
        Vector wi;
        float pdf;
        VisibilityTester vis;
        Spectrum Ls = light.Sample_L(Point(r[0], r[1], r[2]), r[3], ls, 0.f, &wi, &pdf, &vis);
        float c[3];
        Ls.ToRGB(c);
        float* o = out + 16 * i;
        o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
        o[3] = wi.x; o[4] = wi.y; o[5] = wi.z;
        o[6] = pdf;
        o[7] = vis.r.o.x; o[8] = vis.r.o.y; o[9] = vis.r.o.z;
        o[10] = vis.r.d.x; o[11] = vis.r.d.y; o[12] = vis.r.d.z;
        o[13] = vis.r.mint; o[14] = vis.r.maxt; o[15] = 0.f;
    }
}

}  // extern "C"
