"""Many ray-bvh scenes in one launch (pbg_sceneset_* in include/pbrt_gb300.h).

The reference answers one scene's ray batch per call (core/scene.cpp:69-120
into accelerators/rayBVH.cpp:615-1323); a SceneSet answers the nearest-hit
and any-hit batches of up to 4096 scenes with one persistent kernel.  Rays
and results are device tensors laid out scene after scene:

    set = SceneSet([tris_0, tris_1, ...])
    set.trace(o4n, d4n, near_offsets, prim, t, b1, b2,
              o4s, d4s, occ_offsets, occ)

o4/d4 are float32 [n, 4] CUDA tensors (origin, mint) / (direction, maxt);
offsets are host int64 arrays of nscenes + 1 entries (scene k owns rays
offsets[k] .. offsets[k+1]); prim is int32 (local triangle index, -1 =
miss), t/b1/b2 float32, occ uint8.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class BatchParams(C.Structure):
    _fields_ = [("tile", C.c_int32), ("ctas_per_sm", C.c_int32), ("threads", C.c_int32),
                ("use_graph", C.c_int32), ("walk", C.c_int32), ("reserved", C.c_int32 * 7)]


class BatchStats(C.Structure):
    _fields_ = [("ms", C.c_double), ("scene_ms_p50", C.c_double), ("scene_ms_p99", C.c_double),
                ("rays", C.c_uint64), ("tile", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("threads", C.c_int32), ("graph_replayed", C.c_int32), ("walk", C.c_int32),
                ("reserved", C.c_int32)]


_bound = False


def _bind():
    global _bound
    lib = L.lib()
    if _bound:
        return lib
    vp = C.c_void_p
    lib.pbg_sceneset_create.argtypes = [C.c_int32, vp, vp, C.c_int32, C.POINTER(vp)]
    lib.pbg_sceneset_destroy.argtypes = [vp]
    lib.pbg_sceneset_destroy.restype = None
    lib.pbg_sceneset_trace.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                       C.POINTER(BatchParams), C.POINTER(BatchStats), vp, vp]
    lib.pbg_sceneset_autotune.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                          C.POINTER(BatchParams), vp]
    _bound = True
    return lib


def _ptr(x):
    return None if x is None else x.data_ptr()


def _offsets(off, n):
    if off is None:
        return None
    a = np.ascontiguousarray(np.asarray(off, np.int64))
    if a.shape != (n + 1,):
        raise ValueError(f"offsets need {n + 1} entries, got {a.shape}")
    return a


class SceneSet:
    def __init__(self, scenes, device: int = 0):
        lib = _bind()
        self.tris = [np.ascontiguousarray(np.asarray(t, np.float32).reshape(-1, 9)) for t in scenes]
        n = len(self.tris)
        ptrs = (C.c_void_p * n)(*[t.ctypes.data if len(t) else None for t in self.tris])
        counts = (C.c_int64 * n)(*[len(t) for t in self.tris])
        self.nscenes = n
        self.handle = C.c_void_p()
        L.check(lib.pbg_sceneset_create(n, ptrs, counts, device, C.byref(self.handle)),
                "pbg_sceneset_create")

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            L.lib().pbg_sceneset_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _args(self, o4n, d4n, near_offsets, prim, t, b1, b2, o4s, d4s, occ_offsets, occ):
        no = _offsets(near_offsets, self.nscenes)
        so = _offsets(occ_offsets, self.nscenes)
        self._keep = (no, so)
        return [_ptr(o4n), _ptr(d4n), None if no is None else no.ctypes.data, _ptr(prim), _ptr(t),
                _ptr(b1), _ptr(b2), _ptr(o4s), _ptr(d4s), None if so is None else so.ctypes.data,
                _ptr(occ)]

    def trace(self, o4n=None, d4n=None, near_offsets=None, prim=None, t=None, b1=None, b2=None,
              o4s=None, d4s=None, occ_offsets=None, occ=None, tile=0, ctas_per_sm=0, threads=0,
              use_graph=True, walk=0, stats=False, stream=None):
        """One launch over every scene; returns (stats dict, per-scene ms) when
        stats is set (which synchronises), else None."""
        args = self._args(o4n, d4n, near_offsets, prim, t, b1, b2, o4s, d4s, occ_offsets, occ)
        p = BatchParams(tile, ctas_per_sm, threads, int(bool(use_graph)), walk)
        st = BatchStats()
        per = np.zeros(self.nscenes, np.float64) if stats else None
        L.check(_bind().pbg_sceneset_trace(
            self.handle, *args, C.byref(p), C.byref(st) if stats else None,
            None if per is None else per.ctypes.data,
            None if stream is None else stream.cuda_stream), "pbg_sceneset_trace")
        if not stats:
            return None
        return ({"ms": st.ms, "scene_ms_p50": st.scene_ms_p50, "scene_ms_p99": st.scene_ms_p99,
                 "rays": st.rays, "tile": st.tile, "ctas_per_sm": st.ctas_per_sm,
                 "threads": st.threads, "graph_replayed": bool(st.graph_replayed),
                 "walk": st.walk}, per)

    def trace_host(self, host: dict, dev: dict, near_offsets, occ_offsets, stream, copy_stream,
                   split: int | None = None):
        """Pinned host rays in and results out, in two halves of the scenes:
        the second half's rays are copied while the first half is traced, and
        the first half's results while the second is.  `host` and `dev` map
        o4n, d4n, o4s, d4s, prim, t, b1, b2, occ to pinned host tensors and
        device tensors of the same shapes.  Each half is one trace call over
        every scene, the other half's scenes given empty ranges, so the
        results are those of one call (the graph cache keeps both halves'
        segment tables).  `split` = the first scene of the second half
        (default: where half of the rays are)."""
        import torch
        n = self.nscenes
        no = _offsets(near_offsets, n)
        so = _offsets(occ_offsets, n)
        tot = no + so
        k = split if split is not None else int(np.searchsorted(tot, tot[-1] / 2))
        k = min(max(k, 1), n - 1) if n > 1 else n
        parts = []
        for lo_s, hi_s in ((0, k), (k, n)):
            nb, ne = int(no[lo_s]), int(no[hi_s])
            sb, se = int(so[lo_s]), int(so[hi_s])
            # this part's scenes keep their ranges, relative to its first ray
            pn = np.clip(no - nb, 0, ne - nb)
            ps = np.clip(so - sb, 0, se - sb)
            parts.append((nb, ne, sb, se, pn, ps))
        ev_in = [torch.cuda.Event() for _ in parts]
        ev_done = [torch.cuda.Event() for _ in parts]
        with torch.cuda.stream(copy_stream):
            for (nb, ne, sb, se, _, _), ev in zip(parts, ev_in):
                for key in ("o4n", "d4n"):
                    dev[key][nb:ne].copy_(host[key][nb:ne], non_blocking=True)
                for key in ("o4s", "d4s"):
                    dev[key][sb:se].copy_(host[key][sb:se], non_blocking=True)
                ev.record(copy_stream)
        for (nb, ne, sb, se, pn, ps), ei, ed in zip(parts, ev_in, ev_done):
            stream.wait_event(ei)
            with torch.cuda.stream(stream):
                self.trace(o4n=dev["o4n"][nb:], d4n=dev["d4n"][nb:], near_offsets=pn,
                           prim=dev["prim"][nb:], t=dev["t"][nb:], b1=dev["b1"][nb:], b2=dev["b2"][nb:],
                           o4s=dev["o4s"][sb:], d4s=dev["d4s"][sb:], occ_offsets=ps, occ=dev["occ"][sb:],
                           stream=stream)
            ed.record(stream)
            copy_stream.wait_event(ed)
            with torch.cuda.stream(copy_stream):
                for key in ("prim", "t", "b1", "b2"):
                    host[key][nb:ne].copy_(dev[key][nb:ne], non_blocking=True)
                host["occ"][sb:se].copy_(dev["occ"][sb:se], non_blocking=True)
        copy_stream.synchronize()
        stream.synchronize()

    def autotune(self, o4n=None, d4n=None, near_offsets=None, prim=None, t=None, b1=None, b2=None,
                 o4s=None, d4s=None, occ_offsets=None, occ=None, stream=None) -> dict:
        args = self._args(o4n, d4n, near_offsets, prim, t, b1, b2, o4s, d4s, occ_offsets, occ)
        best = BatchParams()
        L.check(_bind().pbg_sceneset_autotune(
            self.handle, *args, C.byref(best), None if stream is None else stream.cuda_stream),
            "pbg_sceneset_autotune")
        return {"tile": best.tile, "ctas_per_sm": best.ctas_per_sm, "threads": best.threads,
                "walk": best.walk}
