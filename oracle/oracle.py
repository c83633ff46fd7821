"""ctypes access to the CPU oracle (oracle/_build/liboracle.so) and, where it
was built, to the reference's own CPU classes (oracle/_ref/libpbrtref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.

Arrays follow the ray-batch conventions of the package: triangles [T, 9]
float32, rays [8, N] float32 (ox oy oz dx dy dz mint maxt), hits as
(prim int32 with -1 for a miss, t, b1, b2) and occlusion as uint8 0/1.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libpbrtref.so")

_lib = None
_ref = None

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint8)


def build() -> None:
    """Compile the restatement (and, when the reference tree is present, the
    reference harness)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


def reference_tree() -> str:
    """The reference's source tree: $PBRT_REFERENCE, else a directory named
    "reference" beside the repository checkout."""
    return os.environ.get("PBRT_REFERENCE",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def build_ref() -> bool:
    """Build oracle/_ref/libpbrtref.so from the reference sources; returns
    False when the reference tree is not on this machine."""
    ref = reference_tree()
    if not os.path.isdir(os.path.join(ref, "src", "shapes")):
        return False
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"), f"REF={ref}"])
    return True


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_tri_intersect.restype = C.c_int
        L.orc_tri_intersect.argtypes = [_fp, _fp, _fp, C.c_float, C.c_float, _fp, _fp, _fp]
        L.orc_nearest_brute.argtypes = [_fp, C.c_int64, _fp, C.c_int64, _up, _ip, _fp, _fp, _fp, C.c_int]
        L.orc_anyhit_brute.argtypes = [_fp, C.c_int64, _fp, C.c_int64, _up, _up, C.c_int]
        L.orc_hits_geometry.argtypes = [_fp, _fp, _fp, C.c_int64, _ip, _fp, _fp, _fp, _fp]
        L.orc_bvh_build.restype = C.c_void_p
        L.orc_bvh_build.argtypes = [_fp, C.c_int64, C.c_int]
        L.orc_bvh_build_mode.restype = C.c_void_p
        L.orc_bvh_build_mode.argtypes = [_fp, C.c_int64, C.c_int, C.c_int]
        L.orc_bvh_free.argtypes = [C.c_void_p]
        L.orc_bvh_node_count.restype = C.c_int64
        L.orc_bvh_node_count.argtypes = [C.c_void_p]
        L.orc_bvh_nearest.argtypes = [C.c_void_p, _fp, C.c_int64, _up, _ip, _fp, _fp, _fp, C.c_int]
        L.orc_bvh_anyhit.argtypes = [C.c_void_p, _fp, C.c_int64, _up, _up, C.c_int]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_scene_create.restype = C.c_void_p
        R.ref_scene_create.argtypes = [_fp, C.c_int64, C.c_int, _fp, C.c_int]
        R.ref_scene_destroy.argtypes = [C.c_void_p]
        R.ref_nearest.argtypes = [C.c_void_p, _fp, C.c_int64, C.c_int, _ip, _fp, _fp, _fp, _fp]
        R.ref_anyhit.argtypes = [C.c_void_p, _fp, C.c_int64, C.c_int, _up]
        _ref = R
    return _ref


def _f(a):
    return a.ctypes.data_as(_fp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _u(a):
    return None if a is None else a.ctypes.data_as(_up)


def _prep(tris, rays, valid=None):
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays, np.float32)
    assert rays.ndim == 2 and rays.shape[0] == 8
    if valid is not None:
        valid = np.ascontiguousarray(valid, np.uint8)
    return tris, rays, valid


def nearest(tris, rays, valid=None, threads: int | None = None):
    """Brute force over triangles in index order: pbrt's Triangle::Intersect
    with the aggregate's maxt update.  Returns (prim, t, b1, b2)."""
    tris, rays, valid = _prep(tris, rays, valid)
    n = rays.shape[1]
    prim = np.empty(n, np.int32)
    t, b1, b2 = (np.empty(n, np.float32) for _ in range(3))
    lib().orc_nearest_brute(_f(tris), tris.shape[0], _f(rays), n, _u(valid), _i(prim), _f(t),
                            _f(b1), _f(b2), threads or os.cpu_count() or 1)
    return prim, t, b1, b2


def anyhit(tris, rays, valid=None, threads: int | None = None):
    tris, rays, valid = _prep(tris, rays, valid)
    n = rays.shape[1]
    occ = np.empty(n, np.uint8)
    lib().orc_anyhit_brute(_f(tris), tris.shape[0], _f(rays), n, _u(valid), _u(occ),
                           threads or os.cpu_count() or 1)
    return occ


def hits_geometry(tris, uvs, rays, prim, t, b1, b2):
    """DifferentialGeometry of each hit: [n, 14] = p, dpdu, dpdv, nn, u, v."""
    tris, rays, _ = _prep(tris, rays)
    n = rays.shape[1]
    out = np.empty((n, 14), np.float32)
    uvp = None if uvs is None else _f(np.ascontiguousarray(uvs, np.float32))
    lib().orc_hits_geometry(_f(tris), uvp, _f(rays), n, _i(np.ascontiguousarray(prim, np.int32)),
                            _f(np.ascontiguousarray(t, np.float32)),
                            _f(np.ascontiguousarray(b1, np.float32)),
                            _f(np.ascontiguousarray(b2, np.float32)), _f(out))
    return out


def tri_intersect(tri9, o, d, mint, maxt):
    tri9 = np.ascontiguousarray(tri9, np.float32)
    o = np.ascontiguousarray(o, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    t, b1, b2 = C.c_float(), C.c_float(), C.c_float()
    hit = lib().orc_tri_intersect(_f(tri9), _f(o), _f(d), mint, maxt, C.byref(t), C.byref(b1),
                                  C.byref(b2))
    return bool(hit), t.value, b1.value, b2.value


class BVH:
    """The timed CPU baseline: SAH BVH in the manner of pbrt's BVHAccel with
    a conservative box test, so answers equal the brute-force loop."""

    def __init__(self, tris, maxprims: int = 4, box_degenerate: bool = False):
        """box_degenerate: degenerate triangles go into the tree with their
        own boxes, as pbrt's BVHAccel puts them (answers then equal
        BVHAccel's rather than the all-pairs loop's)."""
        self.tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        self.h = lib().orc_bvh_build_mode(_f(self.tris), self.tris.shape[0], maxprims, int(box_degenerate))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_bvh_free(self.h)
            self.h = None

    def nearest(self, rays, valid=None, threads: int | None = None):
        _, rays, valid = _prep(self.tris, rays, valid)
        n = rays.shape[1]
        prim = np.empty(n, np.int32)
        t, b1, b2 = (np.empty(n, np.float32) for _ in range(3))
        lib().orc_bvh_nearest(self.h, _f(rays), n, _u(valid), _i(prim), _f(t), _f(b1), _f(b2),
                              threads or os.cpu_count() or 1)
        return prim, t, b1, b2

    def anyhit(self, rays, valid=None, threads: int | None = None):
        _, rays, valid = _prep(self.tris, rays, valid)
        n = rays.shape[1]
        occ = np.empty(n, np.uint8)
        lib().orc_bvh_anyhit(self.h, _f(rays), n, _u(valid), _u(occ),
                             threads or os.cpu_count() or 1)
        return occ


class _Cam(C.Structure):
    _fields_ = [("r2c", C.c_float * 16), ("c2w", C.c_float * 16), ("xres", C.c_int), ("yres", C.c_int)]


class _Light(C.Structure):
    _fields_ = [("type", C.c_int), ("nsamples", C.c_int), ("pos", C.c_float * 3),
                ("I", C.c_float * 3), ("quad", C.c_float * 12), ("L", C.c_float * 3),
                ("first_tri", C.c_int), ("ntri", C.c_int)]


class _Params(C.Structure):
    _fields_ = [("integrator", C.c_int), ("spp_x", C.c_int), ("spp_y", C.c_int), ("jitter", C.c_int),
                ("max_depth", C.c_int), ("seed", C.c_uint64), ("albedo", C.c_float * 3)]


def _render_structs(r2c, c2w, xres, yres, lights, integrator, spp, jitter, max_depth, seed, albedo):
    cam = _Cam()
    cam.r2c[:] = [float(x) for x in np.asarray(r2c, np.float32).reshape(16)]
    cam.c2w[:] = [float(x) for x in np.asarray(c2w, np.float32).reshape(16)]
    cam.xres, cam.yres = int(xres), int(yres)
    arr = (_Light * max(1, len(lights)))()
    for k, lt in enumerate(lights):
        if lt["type"] == "point":
            arr[k].type, arr[k].nsamples = 0, 1
            arr[k].pos[:] = [float(x) for x in lt["pos"]]
            arr[k].I[:] = [float(x) for x in lt["I"]]
        elif lt["type"] == "mesh":
            arr[k].type, arr[k].nsamples = 2, int(lt.get("nsamples", 1))
            arr[k].first_tri, arr[k].ntri = int(lt["first"]), int(lt["ntri"])
            arr[k].L[:] = [float(x) for x in lt["L"]]
        else:
            arr[k].type, arr[k].nsamples = 1, int(lt.get("nsamples", 4))
            arr[k].quad[:] = [float(x) for x in np.asarray(lt["quad"], np.float32).reshape(12)]
            arr[k].L[:] = [float(x) for x in lt["L"]]
    p = _Params()
    p.integrator = {"directlighting": 0, "path": 1}[integrator]
    p.spp_x, p.spp_y = spp
    p.jitter = int(bool(jitter))
    p.max_depth = max_depth
    p.seed = seed
    p.albedo[:] = [float(a) for a in albedo]
    return cam, arr, p


def render(tris, r2c, c2w, xres, yres, lights, integrator="directlighting", spp=(1, 1),
           jitter=False, max_depth=5, seed=1, albedo=(0.7, 0.7, 0.7), threads=None):
    """The CPU restatement of the renderer (oracle/render_oracle.c).  lights:
    dicts {"type": "point", "pos", "I"}, {"type": "quad", "quad", "L",
    "nsamples"} or {"type": "mesh", "first", "ntri", "L", "nsamples"} (the
    scene's triangles [first, first + ntri) as an area light).  Returns rgb
    [yres, xres, 3]."""
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    cam, arr, p = _render_structs(r2c, c2w, xres, yres, lights, integrator, spp, jitter, max_depth,
                                  seed, albedo)
    L = lib()
    L.orc_render.argtypes = [_fp, C.c_int64, C.POINTER(_Cam), C.POINTER(_Light), C.c_int,
                             C.POINTER(_Params), _fp, C.c_int]
    img = np.empty((yres, xres, 3), np.float32)
    L.orc_render(_f(tris), tris.shape[0], C.byref(cam), arr, len(lights), C.byref(p), _f(img),
                 threads or os.cpu_count() or 1)
    return img


def render_stream(tris, r2c, c2w, xres, yres, lights, integrator, image_xy, dims, rng, max_depth=5,
                  albedo=(0.7, 0.7, 0.7), threads=None):
    """The renderer restatement fed one task's reference sample values
    (orc_render_stream; the layout of pbg_sample_stream)."""
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    image_xy = np.ascontiguousarray(image_xy, np.float32)
    dims = np.ascontiguousarray(dims, np.float32)
    rng = np.ascontiguousarray(rng, np.float32)
    cam, arr, p = _render_structs(r2c, c2w, xres, yres, lights, integrator, (1, 1), True, max_depth, 0, albedo)
    L = lib()
    L.orc_render_stream.restype = C.c_int
    L.orc_render_stream.argtypes = [_fp, C.c_int64, C.POINTER(_Cam), C.POINTER(_Light), C.c_int,
                                    C.POINTER(_Params), C.c_int64, _fp, _fp, C.c_int, _fp, C.c_int64, _fp,
                                    C.c_int]
    img = np.empty((yres, xres, 3), np.float32)
    rc = L.orc_render_stream(_f(tris), tris.shape[0], C.byref(cam), arr, len(lights), C.byref(p),
                             image_xy.shape[0], _f(image_xy), _f(dims), dims.shape[1], _f(rng), rng.shape[0],
                             _f(img), threads or os.cpu_count() or 1)
    if rc != 0:
        raise ValueError("orc_render_stream: bad stream")
    return img


class RenderCounter:
    """The CPU restatement of a frame, for timing: the BVH is built once;
    count(first, stride) traces the samples first, first + stride, ... of the
    frame (every ray a whole path of the GPU frame would trace) and returns
    (nearest-hit rays, shadow rays)."""

    def __init__(self, tris, r2c, c2w, xres, yres, lights, integrator="path", spp=(1, 1),
                 jitter=True, max_depth=5, seed=1, albedo=(0.7, 0.7, 0.7)):
        self.tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        self.cam, self.arr, self.p = _render_structs(r2c, c2w, xres, yres, lights, integrator, spp,
                                                     jitter, max_depth, seed, albedo)
        self.nlights = len(lights)
        self.samples = int(xres) * int(yres) * int(spp[0]) * int(spp[1])
        L = lib()
        L.orc_render_bvh.restype = C.c_void_p
        L.orc_render_bvh.argtypes = [_fp, C.c_int64]
        L.orc_render_bvh_free.argtypes = [C.c_void_p]
        L.orc_render_count.argtypes = [_fp, C.c_void_p, C.POINTER(_Cam), C.POINTER(_Light), C.c_int,
                                       C.POINTER(_Params), C.c_int64, C.c_int64, C.c_int,
                                       C.POINTER(C.c_uint64)]
        self._L = L
        self.h = L.orc_render_bvh(_f(self.tris), self.tris.shape[0])

    def __del__(self):
        if getattr(self, "h", None):
            self._L.orc_render_bvh_free(self.h)
            self.h = None

    def count(self, first: int, stride: int, threads: int | None = None, seed: int | None = None):
        if seed is not None:
            self.p.seed = int(seed)
        out = (C.c_uint64 * 2)()
        self._L.orc_render_count(_f(self.tris), self.h, C.byref(self.cam), self.arr, self.nlights,
                                 C.byref(self.p), int(first), int(stride),
                                 threads or os.cpu_count() or 1, out)
        return int(out[0]), int(out[1])


def pbrt_task_samples(extent, spp, n1d, n2d, count, nrng, jitter=True, task=0, reference=False):
    """One breadth-first render task's samples as pbrt draws them: RNG(task),
    the stratified sampler over the pixel extent (x0, x1, y0, y1), spp =
    (xsamples, ysamples), the integrators' 1-D / 2-D array sizes n1d / n2d
    in request order; then nrng further RandomFloat draws.  reference=True
    runs pbrt's own sampler (oracle/_ref), else the restatement
    (oracle/pbrt_sampler.c).  Returns (image_xy [n, 2], oned [n, sum n1d],
    twod [n, sum n2d, 2], rng [nrng])."""
    n1d = np.ascontiguousarray(n1d, np.int32)
    n2d = np.ascontiguousarray(n2d, np.int32)
    img = np.zeros((count, 2), np.float32)
    o1 = np.zeros((count, max(1, int(n1d.sum()))), np.float32)
    o2 = np.zeros((count, max(1, int(n2d.sum())), 2), np.float32)
    rr = np.zeros(max(1, nrng), np.float32)
    if reference:
        L = ref()
        fn = L.ref_task_samples
    else:
        L = lib()
        fn = L.orc_pbrt_task_samples
    fn.restype = C.c_int64
    fn.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _ip, C.c_int,
                   _ip, C.c_int, C.c_int64, _fp, _fp, _fp, C.c_int64, _fp]
    x0, x1, y0, y1 = extent
    got = fn(task, x0, x1, y0, y1, spp[0], spp[1], int(bool(jitter)), _i(n1d), len(n1d), _i(n2d), len(n2d),
             count, _f(img), _f(o1), _f(o2), nrng, _f(rr))
    return img[:got], o1[:got, :int(n1d.sum())], o2[:got, :int(n2d.sum())], rr[:nrng]


def area_light_sample(tris, L, q, reference=False):
    """DiffuseAreaLight::Sample_L over the emitter triangles tris [n, 9] for
    rows q [m, 7] = (p.xyz, pEpsilon, uPos[0], uPos[1], uComponent): rows of
    (L.rgb, wi.xyz, pdf, shadow ray o.xyz, d.xyz, mint, maxt, 0).  reference=
    True runs pbrt's own light (oracle/_ref), else the restatement."""
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    q = np.ascontiguousarray(q, np.float32).reshape(-1, 7)
    L3 = np.ascontiguousarray(L, np.float32)
    out = np.zeros((q.shape[0], 16), np.float32)
    fn = ref().ref_area_light_sample if reference else lib().orc_area_light_sample
    fn.argtypes = [_fp, C.c_int, _fp, _fp, C.c_int64, _fp]
    fn(_f(tris), tris.shape[0], _f(L3), _f(q), q.shape[0], _f(out))
    return out


def ref_camera(xres, yres, eye, look, up, fov, xy):
    """The reference's PerspectiveCamera: (r2c [4,4], c2w [4,4], rays [n, 6])
    for raster samples xy [n, 2]."""
    R = ref()
    R.ref_camera.argtypes = [C.c_int, C.c_int, _fp, _fp, _fp, C.c_float, _fp, _fp, _fp, C.c_int64, _fp]
    e = np.asarray(eye, np.float32)
    lk = np.asarray(look, np.float32)
    u = np.asarray(up, np.float32)
    xy = np.ascontiguousarray(xy, np.float32)
    r2c = np.empty(16, np.float32)
    c2w = np.empty(16, np.float32)
    rays = np.empty((len(xy), 6), np.float32)
    R.ref_camera(xres, yres, _f(e), _f(lk), _f(u), fov, _f(r2c), _f(c2w), _f(xy), len(xy), _f(rays))
    return r2c.reshape(4, 4), c2w.reshape(4, 4), rays


def ref_render(scene_text: str, workdir: str):
    """Renders a scene file with the reference's own CPU renderer
    (oracle/_ref/pbrt_ref); returns the PFM image [yres, xres, 3]."""
    exe = os.path.join(HERE, "_ref", "pbrt_ref")
    path = os.path.join(workdir, "scene.pbrt")
    with open(path, "w") as f:
        f.write(scene_text)
    subprocess.check_call([exe, path], cwd=workdir, stdout=subprocess.DEVNULL,
                          stderr=subprocess.DEVNULL)
    return read_pfm(os.path.join(workdir, "out.pfm"))


def read_pfm(path):
    data = open(path, "rb").read()
    parts = data.split(b"\n", 3)
    w, h = (int(x) for x in parts[1].split())
    return np.frombuffer(parts[3], np.float32, count=w * h * 3).reshape(h, w, 3).copy()


class RefScene:
    """The reference's own TriangleMesh + GeometricPrimitive (+ BVHAccel)."""

    def __init__(self, tris, uv_mode: int = 1, uvs=None, bvh_maxprims: int = 4):
        self.tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        self.uvs = None if uvs is None else np.ascontiguousarray(uvs, np.float32)
        self.h = ref().ref_scene_create(_f(self.tris), self.tris.shape[0], uv_mode,
                                        None if self.uvs is None else _f(self.uvs), bvh_maxprims)

    def __del__(self):
        if getattr(self, "h", None):
            ref().ref_scene_destroy(self.h)
            self.h = None

    def nearest(self, rays, use_bvh: bool = False, geometry: bool = False):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[1]
        prim = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        geo = np.empty((n, 14), np.float32) if geometry else None
        ref().ref_nearest(self.h, _f(rays), n, int(use_bvh), _i(prim), _f(t), _f(u), _f(v),
                          None if geo is None else _f(geo))
        return (prim, t, u, v, geo) if geometry else (prim, t, u, v)

    def anyhit(self, rays, use_bvh: bool = False):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[1]
        occ = np.empty(n, np.uint8)
        ref().ref_anyhit(self.h, _f(rays), n, int(use_bvh), _u(occ))
        return occ
