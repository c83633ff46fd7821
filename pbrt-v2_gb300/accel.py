"""Host-side mirror of the reference's batch accelerators.

The pbrt-v2 fork selects its GPU accelerators by scene-file name
(``Accelerator "naive" | "rayhierarchy" | "ray-bvh"``, core/api.cpp:586-591)
and drives them through ``Scene``'s batch dispatch (core/scene.h:71-99,
core/scene.cpp:54-120).  The classes here keep those names and that calling
convention over the C ABI of libpbrtgb300.so:

  NaiveAccel      accelerators/naive.h:15-110      (CreateNaiveAccelerator)
  RayHieararchy   accelerators/rayhierarchy.h      (CreateRayHieararchy, sic)
  RayBVH          accelerators/rayBVH.h            (CreateRayBVH)

Batch methods:
  MaxRaysPerCall()                 -> int (naive.cpp:127-142)
  Preprocess(camera, spp, nx, ny)  tile geometry (rayhierarchy.cpp:250-265)
  Intersect(rays, hit=None, bounce=None)
      rays: [8, n] float32 host array (o.xyz, d.xyz, mint, maxt).  Primary
      form (bounce None): `hit` is output only.  Bounce form: `hit` is in/out,
      rays with hit False are skipped (rayhierarchy.cpp:602-813).  Like the
      reference, maxt of every hit ray is set to its t
      (``r[i].maxt = t``, rayhierarchy.cpp:1126).  Returns (prim, t, b1, b2).
  IntersectP(rays, hit=None)      -> occluded chars b'0'/b'1' per ray
      (naive.cpp:357-437; invalid rays report '0').
Errors raise PbgError carrying the C status (the reference aborts through
Severe(), core/error.cpp:130).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Aggregate:
    kind = None

    def __init__(self, tris, uvs=None, params: L.Params | None = None):
        self.tris = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 9))
        self.uvs = None if uvs is None else np.ascontiguousarray(np.asarray(uvs, np.float32).reshape(-1, 6))
        self.params = params or L.Params()
        self.handle = C.c_void_p()
        lib = L.lib()
        L.check(lib.pbg_scene_create(self.tris.ctypes.data if len(self.tris) else None,
                                     None if self.uvs is None else self.uvs.ctypes.data,
                                     len(self.tris), L.ACCEL[self.kind], C.byref(self.params),
                                     C.byref(self.handle)), "pbg_scene_create")
        self.tile = None

    @classmethod
    def from_mesh(cls, P, indices, uv=None, params: L.Params | None = None):
        """The scene from pbrt's TriangleMesh arrays (pbg_scene_create_mesh):
        positions [nverts, 3], vertex indices [ntri, 3], per-vertex uvs
        [nverts, 2] or None; the triangles are gathered on the device."""
        self = cls.__new__(cls)
        P = np.ascontiguousarray(np.asarray(P, np.float32).reshape(-1, 3))
        vi = np.ascontiguousarray(np.asarray(indices, np.int32).reshape(-1, 3))
        uvv = None if uv is None else np.ascontiguousarray(np.asarray(uv, np.float32).reshape(-1, 2))
        self.params = params or L.Params()
        self.handle = C.c_void_p()
        self.tile = None
        # the library checks the indices; the host copies below come after
        L.check(L.lib().pbg_scene_create_mesh(P.ctypes.data if len(P) else None, len(P),
                                              vi.ctypes.data if len(vi) else None, len(vi),
                                              None if uvv is None else uvv.ctypes.data, L.ACCEL[cls.kind],
                                              C.byref(self.params), C.byref(self.handle)), "pbg_scene_create_mesh")
        self.tris = np.ascontiguousarray(P[vi].reshape(-1, 9)) if len(vi) else np.zeros((0, 9), np.float32)
        self.uvs = None if uvv is None else np.ascontiguousarray(uvv[vi].reshape(-1, 6))
        return self

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            L.lib().pbg_scene_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- reference-facing batch API ------------------------------------

    def MaxRaysPerCall(self) -> int:
        v = C.c_int64()
        L.check(L.lib().pbg_max_rays_per_call(self.handle, C.byref(v)), "pbg_max_rays_per_call")
        return int(v.value)

    def Preprocess(self, camera=None, samplesPerPixel: int = 1, nx: int = 1, ny: int = 1,
                   xres: int | None = None, yres: int | None = None):
        """Ray-image size of one task tile: W = xRes/nx*spp, H = yRes/ny
        (rayhierarchy.cpp:250-265).  Batches of exactly W*H rays are then
        grouped by 2-D image tiles in the ray hierarchy."""
        if camera is not None and xres is None:
            xres, yres = camera.xres, camera.yres
        if xres is not None and yres is not None:
            self.tile = (xres // nx * samplesPerPixel, yres // ny)
            L.check(L.lib().pbg_preprocess(self.handle, self.tile[0], self.tile[1]),
                    "pbg_preprocess")

    @staticmethod
    def _rays_struct(rays: np.ndarray, valid: np.ndarray | None) -> L.Rays:
        r = L.Rays()
        for k, name in enumerate(("ox", "oy", "oz", "dx", "dy", "dz", "mint", "maxt")):
            setattr(r, name, _fptr(rays[k]))
        r.valid = None if valid is None else valid.ctypes.data_as(C.POINTER(C.c_uint8))
        return r

    def Intersect(self, rays, hit=None, bounce=None):
        rays = np.ascontiguousarray(rays, np.float32) if not (
            isinstance(rays, np.ndarray) and rays.flags.c_contiguous and rays.dtype == np.float32) else rays
        assert rays.ndim == 2 and rays.shape[0] == 8
        n = rays.shape[1]
        valid = None
        if bounce is not None and hit is not None:
            valid = np.ascontiguousarray(np.asarray(hit).astype(np.uint8))
        prim = np.empty(n, np.int32)
        t, b1, b2 = (np.empty(n, np.float32) for _ in range(3))
        h = L.Hits(prim.ctypes.data_as(C.POINTER(C.c_int32)), _fptr(t), _fptr(b1), _fptr(b2))
        rs = self._rays_struct(rays, valid)
        L.check(L.lib().pbg_intersect(self.handle, C.byref(rs), n, C.byref(h)), "pbg_intersect")
        got = prim >= 0
        rays[7, got] = t[got]
        if hit is not None:
            hit[...] = got
        return prim, t, b1, b2

    def IntersectP(self, rays, hit=None) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[1]
        valid = None if hit is None else np.ascontiguousarray(np.asarray(hit).astype(np.uint8))
        occ = np.empty(n, np.uint8)
        rs = self._rays_struct(rays, valid)
        L.check(L.lib().pbg_occluded(self.handle, C.byref(rs), n, occ.ctypes.data), "pbg_occluded")
        return np.where(occ != 0, np.uint8(ord("1")), np.uint8(ord("0"))).astype(np.uint8)

    def HitGeometry(self, rays, prim, t, b1, b2) -> np.ndarray:
        """[n, 14] = p, dpdu, dpdv, nn, u, v (shapes/trianglemesh.cpp:158-190)."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[1]
        prim = np.ascontiguousarray(prim, np.int32)
        t, b1, b2 = (np.ascontiguousarray(x, np.float32) for x in (t, b1, b2))
        out = np.empty((n, 14), np.float32)
        h = L.Hits(prim.ctypes.data_as(C.POINTER(C.c_int32)), _fptr(t), _fptr(b1), _fptr(b2))
        rs = self._rays_struct(rays, None)
        L.check(L.lib().pbg_hit_geometry(self.handle, C.byref(rs), C.byref(h), n, out.ctypes.data),
                "pbg_hit_geometry")
        return out

    # -- device-resident forms (torch tensors) ---------------------------

    def intersect_device(self, o4, d4, prim, t, b1, b2, valid=None, stream=None):
        n = o4.shape[0]
        L.check(L.lib().pbg_intersect_device(
            self.handle, o4.data_ptr(), d4.data_ptr(), None if valid is None else valid.data_ptr(),
            n, prim.data_ptr(), t.data_ptr(), b1.data_ptr(), b2.data_ptr(),
            None if stream is None else stream.cuda_stream), "pbg_intersect_device")

    def autotune(self, o4, d4, anyhit=False, incoherent=False, valid=None, reps=3, stream=None) -> dict:
        """pbg_autotune on a device batch: times every launch shape of this
        accelerator on it, checks that they all give the same results, and
        keeps the fastest.  Returns the candidates' settings and times."""
        r = L.TuneResult()
        query = (1 if anyhit else 0) | (2 if incoherent else 0)
        L.check(L.lib().pbg_autotune(self.handle, o4.data_ptr(), d4.data_ptr(),
                                     None if valid is None else valid.data_ptr(), o4.shape[0], query, reps,
                                     C.byref(r), None if stream is None else stream.cuda_stream),
                "pbg_autotune")
        names = {"naive": ("ctas_per_sm",), "rayhierarchy": ("seed_nodes", "grid_ctas_per_sm"),
                 "ray-bvh": ("walk",)}[self.kind]
        cands = [{"setting": {k: int(r.setting[i][j]) for j, k in enumerate(names)}, "ms": round(float(r.ms[i]), 4)}
                 for i in range(r.ncandidates)]
        return {"candidates": cands, "best": cands[r.best]["setting"], "mismatches": int(r.mismatches)}

    def occluded_device(self, o4, d4, occ, valid=None, stream=None):
        n = o4.shape[0]
        L.check(L.lib().pbg_occluded_device(
            self.handle, o4.data_ptr(), d4.data_ptr(), None if valid is None else valid.data_ptr(),
            n, occ.data_ptr(), None if stream is None else stream.cuda_stream),
            "pbg_occluded_device")

    # -- cluster hints (ray-bvh) ----------------------------------------

    def clusters_of_device(self, prim, cluster, stream=None):
        """cluster[i] (uint16 tensor) = the BVH top-cut cluster of triangle
        prim[i] (0xffff for -1)."""
        L.check(L.lib().pbg_clusters_of_device(self.handle, prim.data_ptr(), prim.shape[0], cluster.data_ptr(),
                                               None if stream is None else stream.cuda_stream),
                "pbg_clusters_of_device")

    def intersect_hinted_device(self, o4, d4, hint, prim, t, b1, b2, valid=None, stream=None):
        L.check(L.lib().pbg_intersect_hinted_device(
            self.handle, o4.data_ptr(), d4.data_ptr(), None if valid is None else valid.data_ptr(), o4.shape[0],
            None if hint is None else hint.data_ptr(), prim.data_ptr(), t.data_ptr(), b1.data_ptr(),
            b2.data_ptr(), None if stream is None else stream.cuda_stream), "pbg_intersect_hinted_device")

    def occluded_hinted_device(self, o4, d4, hint, occ, occluders=None, valid=None, stream=None):
        L.check(L.lib().pbg_occluded_hinted_device(
            self.handle, o4.data_ptr(), d4.data_ptr(), None if valid is None else valid.data_ptr(), o4.shape[0],
            None if hint is None else hint.data_ptr(), occ.data_ptr(),
            None if occluders is None else occluders.data_ptr(), None if stream is None else stream.cuda_stream),
            "pbg_occluded_hinted_device")

    def stats(self) -> dict:
        c = L.Counters()
        L.check(L.lib().pbg_stats(self.handle, C.byref(c)), "pbg_stats")
        return {"rays_nearest": c.rays_nearest, "rays_occluded": c.rays_occluded,
                "calls": c.calls, "bvh_nodes": c.bvh_nodes, "kernel_launches": c.kernel_launches,
                "timed_launches": dict(zip(L.STAGES, list(c.timed_launches))),
                "work": dict(zip(("node_tests", "leaves", "filter_tests", "exact_tests",
                                  "exact_hits", "filter_stage2"), list(c.work))),
                "origin_reuses": c.origin_reuses, "origin_reruns": c.origin_reruns,
                "queue_reruns": c.queue_reruns,
                "stage_ms": dict(zip(L.STAGES, list(c.stage_ms))),
                "wide_nodes": c.wide_nodes, "wide_build_ms": c.wide_build_ms}

    # -- learned traversal ordering (ray-bvh) ------------------------------

    def learn_enable(self, on: bool = True, batch: int = 0, steps_per_train: int = 0, lr: float = 0.0,
                     momentum: float = 0.0, records: int = 0, seed: int = 0,
                     margin: float = 0.0, queries: int = 0) -> None:
        """Builds the BVH clusters and the MLP (pbg_learn_enable); the
        accelerator then collects records from its batches (queries: 1
        nearest-hit first hits, 2 any-hit occluders, 3 / 0 both) and ordered
        walks start once the network has trained."""
        lib = L.lib()
        lib.pbg_learn_enable.argtypes = [C.c_void_p, C.c_int32, C.POINTER(L.LearnParams)]
        p = L.LearnParams()
        p.batch, p.steps_per_train, p.lr, p.momentum = batch, steps_per_train, lr, momentum
        p.records, p.seed, p.margin, p.queries = records, seed, margin, queries
        L.check(lib.pbg_learn_enable(self.handle, int(on), C.byref(p)), "pbg_learn_enable")

    def learn_train(self, steps: int = 0) -> None:
        lib = L.lib()
        lib.pbg_learn_train.argtypes = [C.c_void_p, C.c_int32]
        L.check(lib.pbg_learn_train(self.handle, steps), "pbg_learn_train")

    def learn_stats(self) -> dict:
        lib = L.lib()
        lib.pbg_learn_get_stats.argtypes = [C.c_void_p, C.POINTER(L.LearnStats)]
        s = L.LearnStats()
        L.check(lib.pbg_learn_get_stats(self.handle, C.byref(s)), "pbg_learn_get_stats")
        return {"trained_steps": s.trained_steps, "records": s.records, "last_loss": s.last_loss,
                "last_accuracy": s.last_accuracy, "infer_ms": s.infer_ms, "train_ms": s.train_ms}

    def profile(self, on: bool | int = True) -> None:
        """Per-stage CUDA-event timing (the GPU_TIMES printouts of the
        reference, core/GPUparallel.h:532-538); level 2 also counts
        traversal work (node tests, ray/triangle tests)."""
        L.check(L.lib().pbg_profile(self.handle, int(on)), "pbg_profile")


class NaiveAccel(Aggregate):
    kind = "naive"


class RayHieararchy(Aggregate):
    kind = "rayhierarchy"


class RayBVH(Aggregate):
    kind = "ray-bvh"


def _params_from(ps: dict | None) -> L.Params:
    ps = ps or {}
    p = L.Params()
    p.chunk_x = int(ps.get("chunkXSize", 0))
    p.chunk_y = int(ps.get("chunkYSize", 0))
    p.height = int(ps.get("height", 0))
    p.bvh_height = int(ps.get("BVHheight", 0))
    p.max_bvh_prim = int(ps.get("maxBVHPrim", 0))
    p.device = int(ps.get("device", 0))
    p.ray_sort = int(ps.get("raySort", 0))
    p.rh_cluster_levels = int(ps.get("clusterLevels", 0))
    p.walk = int(ps.get("walk", 0))
    p.bvh_build = int(ps.get("bvhBuild", 0))
    p.rh_queue_pairs = int(ps.get("queuePairs", 0))
    return p


def CreateNaiveAccelerator(tris, ps: dict | None = None, uvs=None) -> NaiveAccel:
    """naive.cpp:440-445 (params onGPU, method: the device path is the only
    path, so both are accepted and ignored)."""
    return NaiveAccel(tris, uvs, _params_from(ps))


def CreateRayHieararchy(tris, ps: dict | None = None, uvs=None) -> RayHieararchy:
    """rayhierarchy.cpp:1329-1348 (chunkXSize, chunkYSize, height, ...)."""
    return RayHieararchy(tris, uvs, _params_from(ps))


def CreateRayBVH(tris, ps: dict | None = None, uvs=None) -> RayBVH:
    """rayBVH.cpp:1326-1344 (BVHheight, maxBVHPrim, ...)."""
    return RayBVH(tris, uvs, _params_from(ps))


def MakeAcceleratorFromMesh(name: str, P, indices, uv=None, ps: dict | None = None) -> Aggregate:
    """MakeAccelerator for a mesh given as pbrt's TriangleMesh arrays."""
    cls = {"naive": NaiveAccel, "rayhierarchy": RayHieararchy, "ray-bvh": RayBVH}.get(name)
    if cls is None:
        raise ValueError(f'Accelerator "{name}" has no batch path')
    return cls.from_mesh(P, indices, uv, _params_from(ps))


def MakeAccelerator(name: str, tris, ps: dict | None = None, uvs=None) -> Aggregate:
    """core/api.cpp:576-594 for the three GPU names; any other name is an
    error, as Scene's batch dispatch raises Severe for other aggregates
    (core/scene.cpp:65)."""
    if name == "naive":
        return CreateNaiveAccelerator(tris, ps, uvs)
    if name == "rayhierarchy":
        return CreateRayHieararchy(tris, ps, uvs)
    if name == "ray-bvh":
        return CreateRayBVH(tris, ps, uvs)
    raise ValueError(f'Accelerator "{name}" has no batch path')
