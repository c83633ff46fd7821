"""The breadth-first renderer on the device (pbg_render) from Python.

Mirrors the reference's scene-file vocabulary: Camera "perspective",
LightSource "point", AreaLightSource "diffuse" on scene triangles (or an
emitter on a parallelogram), Material "matte", SurfaceIntegrator
"directlighting" | "path", Sampler "stratified" (renderers/breadth-first.cpp,
integrators/directlighting.cpp, integrators/path.cpp).  render_stream()
takes the reference's own sample values (one breadth-first task's sampler
output and RNG continuation) in place of the counter-based hash.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L


class Camera(C.Structure):
    _fields_ = [("raster_to_camera", C.c_float * 16), ("camera_to_world", C.c_float * 16),
                ("xres", C.c_int32), ("yres", C.c_int32)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("nsamples", C.c_int32), ("pos", C.c_float * 3),
                ("intensity", C.c_float * 3), ("quad", C.c_float * 12), ("radiance", C.c_float * 3),
                ("first_tri", C.c_int32), ("ntri", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("spp_x", C.c_int32), ("spp_y", C.c_int32),
                ("jitter", C.c_int32), ("max_depth", C.c_int32), ("reserved0", C.c_int32),
                ("seed", C.c_uint64), ("albedo", C.c_float * 3), ("reserved", C.c_int32 * 8)]


class SampleStream(C.Structure):
    _fields_ = [("count", C.c_int64), ("image_xy", C.POINTER(C.c_float)), ("dims", C.POINTER(C.c_float)),
                ("ndims", C.c_int32), ("reserved", C.c_int32), ("rng", C.POINTER(C.c_float)),
                ("nrng", C.c_int64)]


class RenderStats(C.Structure):
    _fields_ = [("camera_rays", C.c_uint64), ("nearest_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("bounces", C.c_uint64), ("ms_total", C.c_double)]


INTEGRATORS = {"directlighting": 0, "path": 1}


def _bind():
    lib = L.lib()
    if not getattr(lib, "_render_bound", False):
        lib.pbg_render.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32,
                                   C.POINTER(RenderParams), C.c_void_p, C.POINTER(RenderStats)]
        lib.pbg_render_stream.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(Light), C.c_int32,
                                          C.POINTER(RenderParams), C.POINTER(SampleStream), C.c_void_p,
                                          C.POINTER(RenderStats)]
        lib._render_bound = True
    return lib


def camera_struct(r2c, c2w, xres: int, yres: int) -> Camera:
    cam = Camera()
    cam.raster_to_camera[:] = [float(x) for x in np.asarray(r2c, np.float32).reshape(16)]
    cam.camera_to_world[:] = [float(x) for x in np.asarray(c2w, np.float32).reshape(16)]
    cam.xres, cam.yres = int(xres), int(yres)
    return cam


def _cross_pbrt(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]]).astype(np.float32)


def _normalize(v):
    v = np.asarray(v, np.float32)
    ln = np.float32(np.sqrt(np.float32(np.float32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])))
    return (v * (np.float32(1.0) / ln)).astype(np.float32)


def perspective_camera(xres: int, yres: int, eye, look, up, fov: float):
    """RasterToCamera and CameraToWorld of Camera "perspective" after LookAt
    (core/transform.cpp LookAt/Perspective, core/camera.cpp:68-88).
    CameraToWorld follows LookAt's float arithmetic; RasterToCamera is
    inverted in double and rounded once, which can differ from pbrt's float
    Gauss-Jordan inverse in the last bit (the tests use the reference's own
    matrices)."""
    pos = np.asarray(eye, np.float32)
    d = _normalize(np.asarray(look, np.float32) - pos)
    left = _normalize(_cross_pbrt(_normalize(up), d))
    new_up = _cross_pbrt(d, left)
    c2w = np.zeros((4, 4), np.float32)
    c2w[0:3, 0] = left
    c2w[0:3, 1] = new_up
    c2w[0:3, 2] = d
    c2w[0:3, 3] = pos
    c2w[3, 3] = 1.0
    n, f = 1e-2, 1000.0
    persp = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, f / (f - n), -f * n / (f - n)], [0, 0, 1, 0]],
                     np.float64)
    inv_tan = 1.0 / math.tan(math.radians(fov) / 2.0)
    cam_to_screen = np.diag([inv_tan, inv_tan, 1.0, 1.0]) @ persp
    frame = xres / yres
    if frame > 1:
        sw = (-frame, frame, -1.0, 1.0)
    else:
        sw = (-1.0, 1.0, -1.0 / frame, 1.0 / frame)
    screen_to_raster = (np.diag([xres, yres, 1.0, 1.0])
                        @ np.diag([1.0 / (sw[1] - sw[0]), 1.0 / (sw[2] - sw[3]), 1.0, 1.0])
                        @ np.array([[1, 0, 0, -sw[0]], [0, 1, 0, -sw[3]], [0, 0, 1, 0], [0, 0, 0, 1]],
                                   np.float64))
    r2c = np.linalg.inv(cam_to_screen) @ np.linalg.inv(screen_to_raster)
    return r2c.astype(np.float32), c2w


def point_light(pos, intensity) -> Light:
    lt = Light()
    lt.type = 0
    lt.nsamples = 1
    lt.pos[:] = [float(x) for x in pos]
    lt.intensity[:] = [float(x) for x in intensity]
    return lt


def quad_light(quad, radiance, nsamples: int = 4) -> Light:
    """Parallelogram emitter: corners p0, p1, p2, p3 with p2 = p1 + p3 - p0;
    emits on the side of (p1 - p0) x (p3 - p0)."""
    lt = Light()
    lt.type = 1
    lt.nsamples = int(nsamples)
    lt.quad[:] = [float(x) for x in np.asarray(quad, np.float32).reshape(12)]
    lt.radiance[:] = [float(x) for x in radiance]
    return lt


def mesh_light(first_tri: int, ntri: int, radiance, nsamples: int = 1) -> Light:
    """AreaLightSource "diffuse" on the scene's triangles [first_tri,
    first_tri + ntri): pbrt's DiffuseAreaLight over their ShapeSet
    (lights/diffuse.cpp), emitting on the side of each triangle's normal."""
    lt = Light()
    lt.type = 2
    lt.nsamples = int(nsamples)
    lt.first_tri, lt.ntri = int(first_tri), int(ntri)
    lt.radiance[:] = [float(x) for x in radiance]
    return lt


def render_params(integrator="directlighting", spp=(1, 1), jitter=False, max_depth=5, seed=1,
                  albedo=(0.7, 0.7, 0.7)) -> RenderParams:
    p = RenderParams()
    p.integrator = INTEGRATORS[integrator]
    p.spp_x, p.spp_y = int(spp[0]), int(spp[1])
    p.jitter = int(bool(jitter))
    p.max_depth = int(max_depth)
    p.seed = int(seed)
    p.albedo[:] = [float(a) for a in albedo]
    return p


PATH_SAMPLE_DEPTH = 3  # integrators/path.h SAMPLE_DEPTH


def sample_arrays(integrator: str, light_nsamples):
    """The 1-D and 2-D sample array sizes the reference's integrators request,
    in request order (Sample::Add1D / Add2D): directlighting's LightSample
    and BSDFSample offsets per light (integrators/directlighting.cpp:45-62),
    the path integrator's four per bounce below SAMPLE_DEPTH
    (integrators/path.cpp:31-38), then the default volume integrator's two
    (integrators/emission.cpp:31-35)."""
    n1d, n2d = [], []
    if integrator == "directlighting":
        for ns in light_nsamples:
            n1d += [ns, ns]
            n2d += [ns, ns]
    else:
        for _ in range(PATH_SAMPLE_DEPTH):
            n1d += [1, 1, 1, 1]
            n2d += [1, 1, 1]
    return n1d + [1, 1], n2d


def stream_dims(integrator: str, light_nsamples, oned, twod):
    """pbg_sample_stream's per-sample values from the reference's sample
    arrays (oned [n, sum n1d], twod [n, sum n2d, 2] in the order of
    sample_arrays)."""
    oned = np.asarray(oned, np.float32)
    twod = np.asarray(twod, np.float32)
    n = oned.shape[0]
    if integrator == "directlighting":
        cols, o1, o2 = [], 0, 0
        for ns in light_nsamples:
            lcomp, bcomp = oned[:, o1:o1 + ns], oned[:, o1 + ns:o1 + 2 * ns]
            lpos, bdir = twod[:, o2:o2 + ns], twod[:, o2 + ns:o2 + 2 * ns]
            for j in range(ns):
                cols += [lpos[:, j, 0], lpos[:, j, 1], lcomp[:, j], bdir[:, j, 0], bdir[:, j, 1], bcomp[:, j]]
            o1 += 2 * ns
            o2 += 2 * ns
    else:
        cols = []
        for b in range(PATH_SAMPLE_DEPTH):
            lcomp, lnum, bcomp, pcomp = (oned[:, 4 * b + k] for k in range(4))
            lpos, bdir, pdir = (twod[:, 3 * b + k] for k in range(3))
            cols += [lnum, lpos[:, 0], lpos[:, 1], lcomp, bdir[:, 0], bdir[:, 1], bcomp, pdir[:, 0], pdir[:, 1],
                     pcomp]
    return np.ascontiguousarray(np.stack(cols, 1) if cols else np.zeros((n, 1)), np.float32)


def render(acc, camera: Camera, lights, params: RenderParams):
    """Renders through the accelerator's scene; returns (rgb [yres, xres, 3],
    stats dict)."""
    lib = _bind()
    lights = list(lights)
    arr = (Light * max(1, len(lights)))(*lights)
    img = np.empty((camera.yres, camera.xres, 3), np.float32)
    st = RenderStats()
    L.check(lib.pbg_render(acc.handle, C.byref(camera), arr, len(lights), C.byref(params),
                           img.ctypes.data, C.byref(st)), "pbg_render")
    return img, {"camera_rays": st.camera_rays, "nearest_rays": st.nearest_rays,
                 "shadow_rays": st.shadow_rays, "bounces": st.bounces, "ms_total": st.ms_total}


def render_stream(acc, camera: Camera, lights, params: RenderParams, image_xy, dims, rng):
    """pbg_render_stream: one task's sample values (image_xy [n, 2], dims
    [n, ndims] as stream_dims lays them out, rng = the task RNG's later
    draws).  Returns (rgb [yres, xres, 3], stats dict)."""
    lib = _bind()
    lights = list(lights)
    arr = (Light * max(1, len(lights)))(*lights)
    image_xy = np.ascontiguousarray(image_xy, np.float32)
    dims = np.ascontiguousarray(dims, np.float32)
    rng = np.ascontiguousarray(rng, np.float32)
    fp = C.POINTER(C.c_float)
    ss = SampleStream(image_xy.shape[0], image_xy.ctypes.data_as(fp), dims.ctypes.data_as(fp), dims.shape[1], 0,
                      rng.ctypes.data_as(fp), rng.shape[0])
    img = np.empty((camera.yres, camera.xres, 3), np.float32)
    st = RenderStats()
    L.check(lib.pbg_render_stream(acc.handle, C.byref(camera), arr, len(lights), C.byref(params), C.byref(ss),
                                  img.ctypes.data, C.byref(st)), "pbg_render_stream")
    return img, {"camera_rays": st.camera_rays, "nearest_rays": st.nearest_rays,
                 "shadow_rays": st.shadow_rays, "bounces": st.bounces, "ms_total": st.ms_total}
