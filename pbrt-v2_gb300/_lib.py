"""ctypes binding of the C ABI in include/pbrt_gb300.h (libpbrtgb300.so).

The shared library is built in tree (``make -C pbrt-v2_gb300``) into
``pbrt-v2_gb300/_build/``.  Loading it never falls back to anything else: a
missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpbrtgb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "pbrt_gb300.h")

PBG_OK = 0
PBG_ERR_INVALID_ARGUMENT = 1
PBG_ERR_CUDA = 2
PBG_ERR_OUT_OF_MEMORY = 3
PBG_ERR_DEVICE_TIMEOUT = 4
PBG_ERR_NO_DEVICE = 5
PBG_ERR_UNSUPPORTED = 6
PBG_ERR_INTERNAL = 7

ACCEL = {"naive": 0, "rayhierarchy": 1, "ray-bvh": 2}


class PbgError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: status {status} ({status_string(status)}): {last_error()}")


class TuneResult(C.Structure):
    _fields_ = [("ncandidates", C.c_int32), ("best", C.c_int32), ("setting", (C.c_int32 * 3) * 16),
                ("ms", C.c_float * 16), ("mismatches", C.c_uint64)]


class Params(C.Structure):
    _fields_ = [("chunk_x", C.c_int32), ("chunk_y", C.c_int32), ("height", C.c_int32),
                ("bvh_height", C.c_int32), ("max_bvh_prim", C.c_int32), ("device", C.c_int32),
                ("ray_sort", C.c_int32), ("rh_cluster_levels", C.c_int32),
                ("walk", C.c_int32), ("bvh_build", C.c_int32), ("rh_queue_pairs", C.c_int32),
                ("reserved", C.c_int32 * 5)]


_fp = C.POINTER(C.c_float)


class Rays(C.Structure):
    _fields_ = [("ox", _fp), ("oy", _fp), ("oz", _fp), ("dx", _fp), ("dy", _fp), ("dz", _fp),
                ("mint", _fp), ("maxt", _fp), ("valid", C.POINTER(C.c_uint8))]


class Hits(C.Structure):
    _fields_ = [("prim", C.POINTER(C.c_int32)), ("t", _fp), ("b1", _fp), ("b2", _fp)]


class Counters(C.Structure):
    _fields_ = [("rays_nearest", C.c_uint64), ("rays_occluded", C.c_uint64),
                ("calls", C.c_uint64), ("bvh_nodes", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("timed_launches", C.c_uint64 * 4), ("work", C.c_uint64 * 6),
                ("origin_reuses", C.c_uint64), ("origin_reruns", C.c_uint64), ("queue_reruns", C.c_uint64),
                ("stage_ms", C.c_double * 4), ("wide_nodes", C.c_uint64), ("wide_build_ms", C.c_double)]


STAGES = ("sort", "build", "traverse", "other")


class LearnParams(C.Structure):
    _fields_ = [("batch", C.c_int32), ("steps_per_train", C.c_int32), ("lr", C.c_float),
                ("momentum", C.c_float), ("records", C.c_int32), ("margin", C.c_float),
                ("seed", C.c_uint64), ("queries", C.c_int32), ("reserved", C.c_int32 * 7)]


class LearnStats(C.Structure):
    _fields_ = [("trained_steps", C.c_uint64), ("records", C.c_uint64), ("last_loss", C.c_float),
                ("last_accuracy", C.c_float), ("infer_ms", C.c_double), ("train_ms", C.c_double)]


_lib = None


def build(jobs: int = 8) -> None:
    subprocess.check_call(["make", "-s", "-j", str(jobs), "-C", HERE])


def exported_symbols_in_header() -> list[str]:
    """Names of every function the public header declares."""
    import re
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(pbg_[a-z0-9_]+)\s*\(", text)))


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run build() (make -C pbrt-v2_gb300)")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.pbg_version.restype = C.c_char_p
    L.pbg_status_string.restype = C.c_char_p
    L.pbg_status_string.argtypes = [C.c_int]
    L.pbg_last_error.restype = C.c_char_p
    L.pbg_device_count.restype = C.c_int
    L.pbg_scene_create.argtypes = [vp, vp, C.c_int64, C.c_int32, C.POINTER(Params), C.POINTER(vp)]
    L.pbg_scene_create_mesh.argtypes = [vp, C.c_int64, vp, C.c_int64, vp, C.c_int32, C.POINTER(Params),
                                        C.POINTER(vp)]
    L.pbg_scene_destroy.argtypes = [vp]
    L.pbg_scene_destroy.restype = None
    L.pbg_max_rays_per_call.argtypes = [vp, C.POINTER(C.c_int64)]
    L.pbg_intersect.argtypes = [vp, C.POINTER(Rays), C.c_int64, C.POINTER(Hits)]
    L.pbg_occluded.argtypes = [vp, C.POINTER(Rays), C.c_int64, vp]
    L.pbg_intersect_device.argtypes = [vp, vp, vp, vp, C.c_int64, vp, vp, vp, vp, vp]
    L.pbg_occluded_device.argtypes = [vp, vp, vp, vp, C.c_int64, vp, vp]
    L.pbg_clusters_of_device.argtypes = [vp, vp, C.c_int64, vp, vp]
    L.pbg_intersect_hinted_device.argtypes = [vp, vp, vp, vp, C.c_int64, vp, vp, vp, vp, vp, vp]
    L.pbg_occluded_hinted_device.argtypes = [vp, vp, vp, vp, C.c_int64, vp, vp, vp, vp]
    L.pbg_hit_geometry.argtypes = [vp, C.POINTER(Rays), C.POINTER(Hits), C.c_int64, vp]
    L.pbg_hit_geometry_device.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int64, vp, vp]
    L.pbg_autotune.argtypes = [vp, vp, vp, vp, C.c_int64, C.c_int32, C.c_int32, C.POINTER(TuneResult), vp]
    L.pbg_stats.argtypes = [vp, C.POINTER(Counters)]
    L.pbg_profile.argtypes = [vp, C.c_int]
    L.pbg_preprocess.argtypes = [vp, C.c_int64, C.c_int64]
    _lib = L
    return L


def status_string(status: int) -> str:
    return lib().pbg_status_string(status).decode()


def last_error() -> str:
    return lib().pbg_last_error().decode()


def check(status: int, what: str) -> None:
    if status != PBG_OK:
        raise PbgError(status, what)
