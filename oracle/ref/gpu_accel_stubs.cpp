// gpu_accel_stubs.cpp -- out-of-line members of the fork's three OpenCL
// accelerators for the CPU-only reference renderer.  Scene's batch dispatch
// (core/scene.h:71-99) dynamic_casts to these classes, so their vtables and
// type information must exist; the CPU reference renders never construct
// them (its scenes use Accelerator "bvh"), and every member aborts through
// Severe if reached.
#include "stdafx.h"
#include "accelerators/naive.h"
#include "accelerators/rayhierarchy.h"
#include "accelerators/rayBVH.h"
#include "paramset.h"

#define PBG_STUB Severe("GPU accelerator stub reached in the CPU reference build")

NaiveAccel::~NaiveAccel() {}
BBox NaiveAccel::WorldBound() const { PBG_STUB; return BBox(); }
unsigned int NaiveAccel::MaxRaysPerCall() { PBG_STUB; return 0; }
void NaiveAccel::Intersect(const RayDifferential*, Intersection*, bool*, const int, const int) { PBG_STUB; }
bool NaiveAccel::Intersect(const Ray&, Intersection*) const { PBG_STUB; return false; }
bool NaiveAccel::IntersectP(const Ray&) const { PBG_STUB; return false; }
void NaiveAccel::IntersectP(const Ray*, char*, const size_t, const bool*) { PBG_STUB; }
NaiveAccel* CreateNaiveAccelerator(const vector<Reference<Primitive> >&, const ParamSet&) { PBG_STUB; return NULL; }

RayHieararchy::~RayHieararchy() {}
BBox RayHieararchy::WorldBound() const { PBG_STUB; return BBox(); }
bool RayHieararchy::Intersect(const Ray&, Intersection*) const { PBG_STUB; return false; }
bool RayHieararchy::IntersectP(const Ray&) const { PBG_STUB; return false; }
unsigned int RayHieararchy::MaxRaysPerCall() { PBG_STUB; return 0; }
void RayHieararchy::Preprocess(const Camera*, const unsigned, const int, const int) { PBG_STUB; }
void RayHieararchy::Intersect(const RayDifferential*, Intersection*, bool*, const unsigned int) { PBG_STUB; }
void RayHieararchy::Intersect(const RayDifferential*, Intersection*, bool*, const unsigned int, const int) { PBG_STUB; }
void RayHieararchy::IntersectP(const Ray*, char*, const size_t, const bool*) { PBG_STUB; }
RayHieararchy* CreateRayHieararchy(const vector<Reference<Primitive> >&, const ParamSet&) { PBG_STUB; return NULL; }

RayBVH::~RayBVH() {}
BBox RayBVH::WorldBound() const { PBG_STUB; return BBox(); }
bool RayBVH::Intersect(const Ray&, Intersection*) const { PBG_STUB; return false; }
bool RayBVH::IntersectP(const Ray&) const { PBG_STUB; return false; }
unsigned int RayBVH::MaxRaysPerCall() { PBG_STUB; return 0; }
void RayBVH::Preprocess() { PBG_STUB; }
void RayBVH::Preprocess(const Camera*, const unsigned, const int, const int) { PBG_STUB; }
void RayBVH::Intersect(const RayDifferential*, Intersection*, bool*, const unsigned int) { PBG_STUB; }
void RayBVH::Intersect(const RayDifferential*, Intersection*, bool*, const unsigned int, const int) { PBG_STUB; }
void RayBVH::IntersectP(const Ray*, char*, const size_t, const bool*) { PBG_STUB; }
RayBVH* CreateRayBVH(const vector<Reference<Primitive> >&, const ParamSet&) { PBG_STUB; return NULL; }
