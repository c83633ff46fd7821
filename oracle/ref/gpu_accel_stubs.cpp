// gpu_accel_stubs.cpp -- a CPU batch backend for the fork's three OpenCL
// accelerators in the reference renderer built from its own sources
// (target pbrt_ref).  TEST INFRASTRUCTURE ONLY.
//
// Scene's batch dispatch (core/scene.h:71-99, core/scene.cpp:54-120)
// dynamic_casts to NaiveAccel, RayHieararchy and RayBVH, and the
// breadth-first renderer (renderers/breadth-first.cpp) only runs through
// that dispatch.  Here each class answers its batch calls with host loops
// over pbrt's own GeometricPrimitive::Intersect / IntersectP (the
// primitives fully refined, tested in index order with pbrt's maxt update:
// the answers of a sequential aggregate), keeping the host-side contract of
// the fork's batch methods (accelerators/naive.cpp:204-338, :357-437;
// rayhierarchy.cpp:602-1326):
//   * batch Intersect: maxt is reset to infinity, a hit sets r[i].maxt = t
//     and fills in[i] (GeometricPrimitive::Intersect sets dg, primitive,
//     transforms, ids and rayEpsilon = 1e-3 t); hit[i] is output only for
//     primary batches, in/out for bounce batches (false = skip the ray);
//   * batch IntersectP: '0' / '1' for every ray, '0' for invalid ones;
//   * MaxRaysPerCall returns 409,600 (rayhierarchy.cpp:309).
// The OpenCL kernels, their parts and repair passes are not reproduced: the
// fork's GPU kernels loosen the triangle test, and pbrt's CPU test is the
// contract the GPU build follows.
#include <map>
#include <pthread.h>

#include "stdafx.h"
#include "accelerators/naive.h"
#include "accelerators/rayhierarchy.h"
#include "accelerators/rayBVH.h"
#include "intersection.h"
#include "paramset.h"

namespace {

struct CpuBatch {
    vector<Reference<Primitive> > prims;
    BBox bound;
};

// The classes' declared members belong to the OpenCL path; the backend keeps
// its own state per accelerator object.
std::map<const void*, CpuBatch*>& table() {
    static std::map<const void*, CpuBatch*> t;
    return t;
}

void attach(const void* self, const vector<Reference<Primitive> >& p) {
    CpuBatch* b = new CpuBatch();
    for (uint32_t i = 0; i < p.size(); ++i) p[i]->FullyRefine(b->prims);
    for (uint32_t i = 0; i < b->prims.size(); ++i) b->bound = Union(b->bound, b->prims[i]->WorldBound());
    table()[self] = b;
}

void detach(const void* self) {
    std::map<const void*, CpuBatch*>::iterator it = table().find(self);
    if (it == table().end()) return;
    delete it->second;
    table().erase(it);
}

const CpuBatch& of(const void* self) {
    std::map<const void*, CpuBatch*>::iterator it = table().find(self);
    if (it == table().end()) Severe("CPU batch backend: accelerator not constructed");
    return *it->second;
}

bool loop_intersect(const CpuBatch& b, const Ray& r, Intersection* in) {
    bool hit = false;
    for (uint32_t k = 0; k < b.prims.size(); ++k)
        if (b.prims[k]->Intersect(r, in)) hit = true;
    return hit;
}

bool loop_occluded(const CpuBatch& b, const Ray& r) {
    for (uint32_t k = 0; k < b.prims.size(); ++k)
        if (b.prims[k]->IntersectP(r)) return true;
    return false;
}

// Rays are independent: a batch is split across host threads.
struct Job {
    const CpuBatch* b;
    const RayDifferential* rd;
    const Ray* r;
    Intersection* in;
    bool* hit;
    const bool* valid;
    char* occ;
    bool masked;
    int begin, end;
};

void* intersect_job(void* arg) {
    Job* j = (Job*)arg;
    for (int i = j->begin; i < j->end; ++i) {
        if (j->masked && !j->hit[i]) continue;
        j->hit[i] = false;
        Ray ray(j->rd[i]);
        ray.maxt = INFINITY;  // the batch path forces maxt to infinity
        if (loop_intersect(*j->b, ray, &j->in[i])) {
            j->rd[i].maxt = ray.maxt;
            j->hit[i] = true;
        }
    }
    return NULL;
}

void* occluded_job(void* arg) {
    Job* j = (Job*)arg;
    for (int i = j->begin; i < j->end; ++i) {
        j->occ[i] = '0';
        if (!j->valid[i]) continue;
        if (loop_occluded(*j->b, j->r[i])) j->occ[i] = '1';
    }
    return NULL;
}

const int kThreads = 8;

void run_jobs(Job proto, int count, void* (*fn)(void*)) {
    Job jobs[kThreads];
    pthread_t th[kThreads];
    const int chunk = (count + kThreads - 1) / kThreads;
    int started = 0;
    for (int k = 0; k < kThreads; ++k) {
        jobs[k] = proto;
        jobs[k].begin = k * chunk;
        jobs[k].end = min(count, (k + 1) * chunk);
        if (jobs[k].begin >= jobs[k].end) break;
        pthread_create(&th[k], NULL, fn, &jobs[k]);
        started = k + 1;
    }
    for (int k = 0; k < started; ++k) pthread_join(th[k], NULL);
}

void batch_intersect(const void* self, const RayDifferential* r, Intersection* in, bool* hit, int count,
                     bool masked) {
    Job j;
    j.b = &of(self);
    j.rd = r;
    j.r = NULL;
    j.in = in;
    j.hit = hit;
    j.valid = NULL;
    j.occ = NULL;
    j.masked = masked;
    run_jobs(j, count, intersect_job);
}

void batch_occluded(const void* self, const Ray* r, char* occ, size_t count, const bool* valid) {
    Job j;
    j.b = &of(self);
    j.rd = NULL;
    j.r = r;
    j.in = NULL;
    j.hit = NULL;
    j.valid = valid;
    j.occ = occ;
    j.masked = false;
    run_jobs(j, (int)count, occluded_job);
}

const unsigned int kMaxRaysPerCall = 409600;

}  // namespace

// --------------------------------------------------------------- NaiveAccel

NaiveAccel::NaiveAccel(const vector<Reference<Primitive> >& p, bool onG, const string& m) {
    onGPU = onG;
    method = m;
    ocl = NULL;
    vertices = NULL;
    uvs = NULL;
    attach(this, p);
    triangleCount = of(this).prims.size();
    bbox = of(this).bound;
}
NaiveAccel::~NaiveAccel() { detach(this); }
BBox NaiveAccel::WorldBound() const { return bbox; }
unsigned int NaiveAccel::MaxRaysPerCall() { return kMaxRaysPerCall; }
void NaiveAccel::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const int count,
                           const int bounce) {
    batch_intersect(this, r, in, hit, count, bounce != 0);
}
bool NaiveAccel::Intersect(const Ray& r, Intersection* in) const { return loop_intersect(of(this), r, in); }
bool NaiveAccel::IntersectP(const Ray& r) const { return loop_occluded(of(this), r); }
void NaiveAccel::IntersectP(const Ray* r, char* occ, const size_t count, const bool* hit) {
    batch_occluded(this, r, occ, count, hit);
}
NaiveAccel* CreateNaiveAccelerator(const vector<Reference<Primitive> >& prims, const ParamSet& ps) {
    return new NaiveAccel(prims, ps.FindOneBool("onGPU", true), ps.FindOneString("method", "TriRay"));
}

// ------------------------------------------------------------ RayHieararchy

RayHieararchy::RayHieararchy(const vector<Reference<Primitive> >& p, bool, int, int, int, string, bool,
                             const string&, const int&, const unsigned int&) {
    attach(this, p);
    bbox = of(this).bound;
}
RayHieararchy::~RayHieararchy() { detach(this); }
BBox RayHieararchy::WorldBound() const { return of(this).bound; }
bool RayHieararchy::Intersect(const Ray& r, Intersection* in) const { return loop_intersect(of(this), r, in); }
bool RayHieararchy::IntersectP(const Ray& r) const { return loop_occluded(of(this), r); }
unsigned int RayHieararchy::MaxRaysPerCall() { return kMaxRaysPerCall; }
void RayHieararchy::Preprocess(const Camera*, const unsigned, const int, const int) {}
void RayHieararchy::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const unsigned int count) {
    batch_intersect(this, r, in, hit, (int)count, false);
}
void RayHieararchy::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const unsigned int count,
                              const int) {
    batch_intersect(this, r, in, hit, (int)count, true);
}
void RayHieararchy::IntersectP(const Ray* r, char* occ, const size_t count, const bool* hit) {
    batch_occluded(this, r, occ, count, hit);
}
RayHieararchy* CreateRayHieararchy(const vector<Reference<Primitive> >& prims, const ParamSet& ps) {
    return new RayHieararchy(prims, ps.FindOneBool("onGPU", true), ps.FindOneInt("chunkXSize", 4),
                             ps.FindOneInt("chunkYSize", 4), ps.FindOneInt("height", 3),
                             ps.FindOneString("node", "box_dir"), ps.FindOneBool("sort", false),
                             ps.FindOneString("splitmethod", "sah"), ps.FindOneInt("maxBVHPrim", 1),
                             (unsigned int)ps.FindOneInt("repairRun", 1));
}

// ------------------------------------------------------------------- RayBVH

RayBVH::RayBVH(const vector<Reference<Primitive> >& p, bool, int, int, int, int, string, int, const string&) {
    attach(this, p);
    bbox = of(this).bound;
}
RayBVH::~RayBVH() { detach(this); }
BBox RayBVH::WorldBound() const { return of(this).bound; }
bool RayBVH::Intersect(const Ray& r, Intersection* in) const { return loop_intersect(of(this), r, in); }
bool RayBVH::IntersectP(const Ray& r) const { return loop_occluded(of(this), r); }
unsigned int RayBVH::MaxRaysPerCall() { return kMaxRaysPerCall; }
void RayBVH::Preprocess() {}
void RayBVH::Preprocess(const Camera*, const unsigned, const int, const int) {}
void RayBVH::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const unsigned int count) {
    batch_intersect(this, r, in, hit, (int)count, false);
}
void RayBVH::Intersect(const RayDifferential* r, Intersection* in, bool* hit, const unsigned int count, const int) {
    batch_intersect(this, r, in, hit, (int)count, true);
}
void RayBVH::IntersectP(const Ray* r, char* occ, const size_t count, const bool* hit) {
    batch_occluded(this, r, occ, count, hit);
}
RayBVH* CreateRayBVH(const vector<Reference<Primitive> >& prims, const ParamSet& ps) {
    return new RayBVH(prims, ps.FindOneBool("onGPU", true), ps.FindOneInt("chunkXSize", 4),
                      ps.FindOneInt("chunkYSize", 4), ps.FindOneInt("height", 3), ps.FindOneInt("BVHheight", 3),
                      ps.FindOneString("node", "box_dir"), ps.FindOneInt("maxBVHPrim", 1),
                      ps.FindOneString("splitmethod", "sah"));
}
