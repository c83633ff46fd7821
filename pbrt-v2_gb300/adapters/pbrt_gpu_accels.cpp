// pbrt_gpu_accels.cpp -- the pbrt-side binding of libpbrtgb300.so.
//
// A drop-in replacement for the fork's accelerators/naive.cpp,
// accelerators/rayhierarchy.cpp, accelerators/rayBVH.cpp and
// core/GPUparallel.cpp: it implements the members of the unchanged class
// declarations (accelerators/naive.h, rayhierarchy.h, rayBVH.h) over the C
// ABI in include/pbrt_gb300.h, so core/scene.h's dynamic_cast dispatch,
// core/api.cpp's factories and the breadth-first renderer keep working
// unmodified.  Build it with the rest of pbrt and link -lpbrtgb300 (the
// "adapter" target of oracle/ref/Makefile does exactly that).
//
// Per object state (the device scene, the refined primitives, host staging
// buffers) lives in a side table keyed by the object, because the class
// layouts are the reference's.  Triangles are packed in refinement order,
// so the library's triangle index is the index into that primitive list,
// which is how the reference deserialises hits (rayhierarchy.cpp:1094-1130).
#include "stdafx.h"
#include "accelerators/naive.h"
#include "accelerators/rayhierarchy.h"
#include "accelerators/rayBVH.h"
#include "camera.h"
#include "film.h"
#include "intersection.h"
#include "paramset.h"
#include "pbrt_gb300.h"

#include <cmath>
#include <map>

namespace {

struct GpuAccel {
    pbg_scene* scene;
    vector<Reference<Primitive> > prims;  // one GeometricPrimitive(Triangle) per index
    vector<const Texture<float>*> alpha;  // the mesh's alpha texture per index, or NULL
    BBox bound;
    vector<float> soa, t, b1, b2, geo;
    vector<int32_t> prim;
    vector<uint8_t> valid, occ;
    GpuAccel() : scene(NULL) {}
};

std::map<const void*, GpuAccel*>& table() {
    static std::map<const void*, GpuAccel*> t;
    return t;
}

GpuAccel* state(const void* self) {
    std::map<const void*, GpuAccel*>::iterator it = table().find(self);
    if (it == table().end()) Severe("GPU accelerator state missing");
    return it->second;
}

void check(int rc, const char* what) {
    if (rc != PBG_OK) Severe("%s failed: %s (%s)", what, pbg_status_string(rc), pbg_last_error());
}

// The refined triangles as pbrt holds them: every TriangleMesh's points once
// (world space), one index triple per triangle in refinement order, and the
// meshes' per-vertex uvs.
struct MeshArrays {
    vector<float> P, uv;
    vector<int32_t> idx;
    int with_uv, without_uv;  // meshes that have / lack uvs
    MeshArrays() : with_uv(0), without_uv(0) {}
};

// Creates the device scene: straight from the mesh arrays (gathered on the
// device) unless the meshes mix explicit uvs with pbrt's per-corner default
// ((0,0), (1,0), (1,1)), which no per-vertex array can hold -- then the
// triangles are packed here as float[9n] + float[6n].
void create_scene(GpuAccel* g, const MeshArrays& m, int kind, const pbg_params& prm) {
    const int64_t n = (int64_t)(m.idx.size() / 3), nv = (int64_t)(m.P.size() / 3);
    if (m.with_uv == 0 || m.without_uv == 0) {
        check(pbg_scene_create_mesh(nv ? &m.P[0] : NULL, nv, n ? &m.idx[0] : NULL, n,
                                    m.with_uv && nv ? &m.uv[0] : NULL, kind, &prm, &g->scene),
              "pbg_scene_create_mesh");
        return;
    }
    vector<float> tri9((size_t)n * 9), uv6((size_t)n * 6);
    static const float d[6] = {0.f, 0.f, 1.f, 0.f, 1.f, 1.f};
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const int32_t v = m.idx[3 * i + k];
            for (int a = 0; a < 3; ++a) tri9[9 * i + 3 * k + a] = m.P[3 * v + a];
            const bool has = m.uv[2 * v] == m.uv[2 * v];  // NaN marks a vertex of a mesh without uvs
            uv6[6 * i + 2 * k] = has ? m.uv[2 * v] : d[2 * k];
            uv6[6 * i + 2 * k + 1] = has ? m.uv[2 * v + 1] : d[2 * k + 1];
        }
    check(pbg_scene_create(n ? &tri9[0] : NULL, n ? &uv6[0] : NULL, n, kind, &prm, &g->scene),
          "pbg_scene_create");
}

// Rays into SoA rows (o.xyz, d.xyz, mint, maxt), the layout pbg_rays reads.
template <typename RayT>
void stage_rays(GpuAccel* g, const RayT* r, size_t count, pbg_rays* rays) {
    g->soa.resize(8 * count);
    float* s = &g->soa[0];
    for (size_t i = 0; i < count; ++i) {
        s[i] = r[i].o.x;
        s[count + i] = r[i].o.y;
        s[2 * count + i] = r[i].o.z;
        s[3 * count + i] = r[i].d.x;
        s[4 * count + i] = r[i].d.y;
        s[5 * count + i] = r[i].d.z;
        s[6 * count + i] = r[i].mint;
        s[7 * count + i] = r[i].maxt;
    }
    rays->ox = s;
    rays->oy = s + count;
    rays->oz = s + 2 * count;
    rays->dx = s + 3 * count;
    rays->dy = s + 4 * count;
    rays->dz = s + 5 * count;
    rays->mint = s + 6 * count;
    rays->maxt = s + 7 * count;
    rays->valid = NULL;
}

// Batch nearest hit + Intersection records, as rayhierarchy.cpp:1094-1130
// fills them; `mask` (may be NULL) skips rays and leaves their records.
void batch_intersect(GpuAccel* g, const RayDifferential* r, Intersection* in, bool* hit,
                     size_t count, const bool* mask) {
    if (count == 0) return;
    pbg_rays rays;
    stage_rays(g, r, count, &rays);
    if (mask) {
        g->valid.resize(count);
        for (size_t i = 0; i < count; ++i) g->valid[i] = mask[i] ? 1 : 0;
        rays.valid = &g->valid[0];
    }
    g->prim.resize(count);
    g->t.resize(count);
    g->b1.resize(count);
    g->b2.resize(count);
    g->geo.resize(14 * count);
    pbg_hits hits = {&g->prim[0], &g->t[0], &g->b1[0], &g->b2[0]};
    check(pbg_intersect(g->scene, &rays, (int64_t)count, &hits), "pbg_intersect");
    check(pbg_hit_geometry(g->scene, &rays, &hits, (int64_t)count, &g->geo[0]), "pbg_hit_geometry");
    for (size_t i = 0; i < count; ++i) {
        if (mask && !mask[i]) continue;
        hit[i] = false;
        const int32_t k = g->prim[i];
        if (k < 0) continue;
        const GeometricPrimitive* p = dynamic_cast<const GeometricPrimitive*>(g->prims[k].GetPtr());
        const Triangle* shape = p ? dynamic_cast<const Triangle*>(p->GetShapePtr()) : NULL;
        if (!shape) continue;
        const float* q = &g->geo[14 * i];
        const float th = g->t[i];
        DifferentialGeometry dg(r[i](th), Vector(q[3], q[4], q[5]), Vector(q[6], q[7], q[8]),
                                Normal(0, 0, 0), Normal(0, 0, 0), q[12], q[13], shape);
        if (g->alpha[k] && g->alpha[k]->Evaluate(dg) == 0.f)
            continue;  // as the reference: an alpha-cut hit is dropped
        in[i].dg = dg;
        in[i].primitive = p;
        in[i].WorldToObject = *shape->WorldToObject;
        in[i].ObjectToWorld = *shape->ObjectToWorld;
        in[i].shapeId = shape->shapeId;
        in[i].primitiveId = p->primitiveId;
        in[i].rayEpsilon = 1e-3f * th;
        r[i].maxt = th;
        hit[i] = true;
    }
}

// Batch any-hit; occluded[i] = '0' / '1' (naive.cpp:357-437).
void batch_occluded(GpuAccel* g, const Ray* r, char* occluded, size_t count, const bool* mask) {
    if (count == 0) return;
    pbg_rays rays;
    stage_rays(g, r, count, &rays);
    if (mask) {
        g->valid.resize(count);
        for (size_t i = 0; i < count; ++i) g->valid[i] = mask[i] ? 1 : 0;
        rays.valid = &g->valid[0];
    }
    g->occ.resize(count);
    check(pbg_occluded(g->scene, &rays, (int64_t)count, &g->occ[0]), "pbg_occluded");
    for (size_t i = 0; i < count; ++i) occluded[i] = g->occ[i] ? '1' : '0';
}

bool single_intersect(GpuAccel* g, const Ray& ray, Intersection* isect) {
    RayDifferential rd(ray);
    bool hit = false;
    batch_intersect(g, &rd, isect, &hit, 1, NULL);
    if (hit) ray.maxt = rd.maxt;
    return hit;
}

bool single_occluded(GpuAccel* g, const Ray& ray) {
    char c = '0';
    batch_occluded(g, &ray, &c, 1, NULL);
    return c == '1';
}

unsigned int max_rays(GpuAccel* g) {
    int64_t v = 0;
    check(pbg_max_rays_per_call(g->scene, &v), "pbg_max_rays_per_call");
    return (unsigned int)v;
}

void preprocess(GpuAccel* g, const Camera* camera, unsigned spp, int nx, int ny) {
    // ray image of one task tile (rayhierarchy.cpp:250-265)
    const int64_t w = (int64_t)(camera->film->xResolution / nx) * spp;
    const int64_t h = camera->film->yResolution / ny;
    check(pbg_preprocess(g->scene, w, h), "pbg_preprocess");
}

void destroy(const void* self) {
    std::map<const void*, GpuAccel*>::iterator it = table().find(self);
    if (it == table().end()) return;
    pbg_scene_destroy(it->second->scene);
    delete it->second;
    table().erase(it);
}

}  // namespace

// Collects the refined triangles in order as mesh arrays; runs inside a
// member function of each accelerator class, which the fork made friends of
// Triangle (shapes/trianglemesh.h:51-53, :102-104) for exactly this access.
#define PBG_COLLECT_TRIANGLES(ACC, PRIMS, ARR, BOX)                                           \
    do {                                                                                \
        for (uint32_t i_ = 0; i_ < (PRIMS).size(); ++i_) (PRIMS)[i_]->FullyRefine((ACC)->prims);   \
        vector<Reference<Primitive> > kept_;                                            \
        std::map<const TriangleMesh*, int32_t> base_;                                   \
        for (size_t i_ = 0; i_ < (ACC)->prims.size(); ++i_) {                             \
            const GeometricPrimitive* gp_ =                                             \
                dynamic_cast<const GeometricPrimitive*>((ACC)->prims[i_].GetPtr());       \
            const Triangle* sh_ = gp_ ? dynamic_cast<const Triangle*>(gp_->GetShapePtr()) : NULL; \
            if (!sh_) continue; /* non-triangles are dropped, as naive.cpp:66-69 */     \
            const TriangleMesh* m_ = sh_->GetMeshPtr();                                 \
            std::map<const TriangleMesh*, int32_t>::iterator b_ = base_.find(m_);       \
            if (b_ == base_.end()) { /* a new mesh: its points (and uvs) once */        \
                b_ = base_.insert(std::make_pair(m_, (int32_t)((ARR).P.size() / 3))).first; \
                for (int v_ = 0; v_ < m_->nverts; ++v_) {                               \
                    (ARR).P.push_back(m_->p[v_].x);                                       \
                    (ARR).P.push_back(m_->p[v_].y);                                       \
                    (ARR).P.push_back(m_->p[v_].z);                                       \
                    (ARR).uv.push_back(m_->uvs ? m_->uvs[2 * v_] : NAN);                  \
                    (ARR).uv.push_back(m_->uvs ? m_->uvs[2 * v_ + 1] : NAN);              \
                }                                                                       \
                if (m_->uvs) ++(ARR).with_uv;                                             \
                else ++(ARR).without_uv;                                                  \
            }                                                                           \
            for (int v_ = 0; v_ < 3; ++v_) {                                            \
                (ARR).idx.push_back(b_->second + sh_->v[v_]);                             \
                (BOX) = Union((BOX), m_->p[sh_->v[v_]]);                            \
            }                                                                           \
            kept_.push_back((ACC)->prims[i_]);                                            \
            (ACC)->alpha.push_back(m_->alphaTexture.GetPtr());                            \
        }                                                                               \
        (ACC)->prims.swap(kept_);                                                         \
    } while (0)

// ----------------------------------------------------------------- naive

NaiveAccel::NaiveAccel(const vector<Reference<Primitive> >& p, bool onG, const string& m) {
    onGPU = onG;
    method = m;
    GpuAccel* g = new GpuAccel();
    MeshArrays mesh;
    PBG_COLLECT_TRIANGLES(g, p, mesh, bbox);
    triangleCount = g->prims.size();
    pbg_params prm;
    memset(&prm, 0, sizeof(prm));
    create_scene(g, mesh, PBG_ACCEL_NAIVE, prm);
    g->bound = bbox;
    table()[this] = g;
}
NaiveAccel::~NaiveAccel() { destroy(this); }
BBox NaiveAccel::WorldBound() const { return bbox; }
unsigned int NaiveAccel::MaxRaysPerCall() { return max_rays(state(this)); }
void NaiveAccel::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const int count,
                           const int bounce) {
    batch_intersect(state(this), r, in, hit, (size_t)count, bounce > 0 ? hit : NULL);
}
bool NaiveAccel::Intersect(const Ray& ray, Intersection* isect) const {
    return single_intersect(state(this), ray, isect);
}
bool NaiveAccel::IntersectP(const Ray& ray) const { return single_occluded(state(this), ray); }
void NaiveAccel::IntersectP(const Ray* ray, char* occluded, const size_t count, const bool* hit) {
    batch_occluded(state(this), ray, occluded, count, hit);
}
NaiveAccel* CreateNaiveAccelerator(const vector<Reference<Primitive> >& prims, const ParamSet& ps) {
    bool onGPU = ps.FindOneBool("onGPU", true);
    string method = ps.FindOneString("method", "TriRay");
    return new NaiveAccel(prims, onGPU, method);
}

// ---------------------------------------------------------- rayhierarchy

RayHieararchy::RayHieararchy(const vector<Reference<Primitive> >& p, bool onG, int chunkX, int chunkY,
                             int height, string node, bool sortVert, const string& sm,
                             const int& maxBVHPrim, const unsigned int& repairRun
#if (defined STAT_RAY_TRIANGLE || defined STAT_PRAY_TRIANGLE)
                             , int scale
#endif
) {
    GpuAccel* g = new GpuAccel();
    MeshArrays mesh;
    PBG_COLLECT_TRIANGLES(g, p, mesh, bbox);
    triangleCount = g->prims.size();
    pbg_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.chunk_x = chunkX;
    prm.chunk_y = chunkY;
    prm.height = height;
    create_scene(g, mesh, PBG_ACCEL_RAYHIERARCHY, prm);
    g->bound = bbox;
    table()[this] = g;
}
RayHieararchy::~RayHieararchy() { destroy(this); }
BBox RayHieararchy::WorldBound() const { return bbox; }
bool RayHieararchy::Intersect(const Ray& ray, Intersection* isect) const {
    return single_intersect(state(this), ray, isect);
}
bool RayHieararchy::IntersectP(const Ray& ray) const { return single_occluded(state(this), ray); }
unsigned int RayHieararchy::MaxRaysPerCall() { return max_rays(state(this)); }
void RayHieararchy::Preprocess(const Camera* camera, const unsigned samplesPerPixel, const int nx,
                               const int ny) {
    preprocess(state(this), camera, samplesPerPixel, nx, ny);
}
void RayHieararchy::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const unsigned int count
#ifdef STAT_RAY_TRIANGLE
                              , Spectrum* Ls
#endif
) {
    batch_intersect(state(this), r, in, hit, count, NULL);
}
void RayHieararchy::Intersect(const RayDifferential* r, Intersection* in, bool* hit,
                              const unsigned int count, const int bounce) {
    batch_intersect(state(this), r, in, hit, count, hit);
}
void RayHieararchy::IntersectP(const Ray* ray, char* occluded, const size_t count, const bool* hit
#ifdef STAT_PRAY_TRIANGLE
                               , Spectrum* Ls
#endif
) {
    batch_occluded(state(this), ray, occluded, count, hit);
}
RayHieararchy* CreateRayHieararchy(const vector<Reference<Primitive> >& prims, const ParamSet& ps) {
    bool onGPU = ps.FindOneBool("onGPU", true);
    bool sortVert = ps.FindOneBool("sort", false);
    int chunkX = ps.FindOneInt("chunkXSize", 4);
    int chunkY = ps.FindOneInt("chunkYSize", 4);
    int height = ps.FindOneInt("height", 3);
    string node = ps.FindOneString("node", "box_dir");
    string splitMethod = ps.FindOneString("splitmethod", "sah");
    int maxBVHPrim = ps.FindOneInt("maxBVHPrim", 1);
    unsigned int repairRun = ps.FindOneInt("repairRun", 1);
    return new RayHieararchy(prims, onGPU, chunkX, chunkY, height, node, sortVert, splitMethod,
                             maxBVHPrim, repairRun
#if (defined STAT_RAY_TRIANGLE || defined STAT_PRAY_TRIANGLE)
                             , ps.FindOneInt("scale", 50)
#endif
    );
}

// ---------------------------------------------------------------- ray-bvh

RayBVH::RayBVH(const vector<Reference<Primitive> >& p, bool onG, int chunkX, int chunkY, int height,
               int BVHheight, string node, int MaxBVHPrim, const string& sm
#if (defined STAT_RAY_TRIANGLE || defined STAT_PRAY_TRIANGLE)
               , int scale
#endif
) {
    GpuAccel* g = new GpuAccel();
    MeshArrays mesh;
    PBG_COLLECT_TRIANGLES(g, p, mesh, bbox);
    triangleCount = g->prims.size();
    pbg_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.chunk_x = chunkX;
    prm.chunk_y = chunkY;
    prm.height = height;
    prm.bvh_height = BVHheight;
    // the scene-file default of 1 triangle per leaf served the OpenCL
    // kernels; below 2 the library's tuned leaf size is used
    prm.max_bvh_prim = MaxBVHPrim > 1 ? MaxBVHPrim : 0;
    create_scene(g, mesh, PBG_ACCEL_RAYBVH, prm);
    g->bound = bbox;
    table()[this] = g;
}
RayBVH::~RayBVH() { destroy(this); }
BBox RayBVH::WorldBound() const { return bbox; }
bool RayBVH::Intersect(const Ray& ray, Intersection* isect) const {
    return single_intersect(state(this), ray, isect);
}
bool RayBVH::IntersectP(const Ray& ray) const { return single_occluded(state(this), ray); }
unsigned int RayBVH::MaxRaysPerCall() { return max_rays(state(this)); }
void RayBVH::Preprocess() {}  // the BVH is built with the scene
void RayBVH::Preprocess(const Camera* camera, const unsigned samplesPerPixel, const int nx,
                        const int ny) {
    preprocess(state(this), camera, samplesPerPixel, nx, ny);
}
void RayBVH::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const unsigned int count
#ifdef STAT_RAY_TRIANGLE
                       , Spectrum* Ls
#endif
) {
    batch_intersect(state(this), r, in, hit, count, NULL);
}
void RayBVH::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const unsigned int count,
                       const int bounce) {
    batch_intersect(state(this), r, in, hit, count, hit);
}
void RayBVH::IntersectP(const Ray* ray, char* occluded, const size_t count, const bool* hit
#ifdef STAT_PRAY_TRIANGLE
                        , Spectrum* Ls
#endif
) {
    batch_occluded(state(this), ray, occluded, count, hit);
}
RayBVH* CreateRayBVH(const vector<Reference<Primitive> >& prims, const ParamSet& ps) {
    bool onGPU = ps.FindOneBool("onGPU", true);
    int chunkX = ps.FindOneInt("chunkXSize", 4);
    int chunkY = ps.FindOneInt("chunkYSize", 4);
    int height = ps.FindOneInt("height", 3);
    int BVHheight = ps.FindOneInt("BVHheight", 3);
    int maxBVHPrim = ps.FindOneInt("maxBVHPrim", 1);
    string node = ps.FindOneString("node", "box_dir");
    string splitMethod = ps.FindOneString("splitmethod", "sah");
    return new RayBVH(prims, onGPU, chunkX, chunkY, height, BVHheight, node, maxBVHPrim, splitMethod
#if (defined STAT_RAY_TRIANGLE || defined STAT_PRAY_TRIANGLE)
                      , ps.FindOneInt("scale", 50)
#endif
    );
}
