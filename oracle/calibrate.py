"""Port-vs-reference calibration of the CPU baseline (test infrastructure).

The CPU baseline that travels with the benchmark is the oracle's C
restatement (oracle/bvh_oracle.c, oracle/render_oracle.c): the reference's
own sources do not exist where the benchmark runs.  This script measures,
on one host thread and on the same rays, how fast that restatement is
against the reference's own code built from its sources (oracle/_ref:
core/shape.cpp, shapes/trianglemesh.cpp, accelerators/bvh.cpp), so that a
CPU figure measured with the port can be read as the reference's:

  * SAH BVH construction of the 1,024,000-triangle displaced-icosphere
    scene (pbrt's BVHAccel with maxprims 4 and the "sah" split against the
    oracle's builder);
  * nearest-hit and any-hit queries on that scene: the 1024x1024 camera
    rays of the path frame, and incoherent rays (uniform origins and
    directions in the scene's box), both through each side's BVH.

Usage:  python oracle/calibrate.py [--rays N]
Prints one JSON line per measurement and a summary table.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# run as a script, this folder is first on the path and its oracle.py would
# shadow the package of the same name
sys.path[0] = ROOT

import pbg_import  # noqa: E402
from oracle import oracle as O  # noqa: E402

pbg_import.load()


def camera_rays(n, seed=0):
    """Camera rays of the path frame (the reference's PerspectiveCamera at
    the frame's eye, 1024x1024), a seeded subset of n raster positions;
    [8, n] rows ox oy oz dx dy dz mint maxt."""
    import bench
    g = np.random.default_rng(seed)
    xy = g.uniform(0, bench.PATH_RES, (n, 2)).astype(np.float32)
    cam = bench.PATH_CAMERA
    _, _, r6 = O.ref_camera(bench.PATH_RES, bench.PATH_RES, cam["eye"], cam["look"], cam["up"],
                            cam["fov"], xy)
    rays = np.empty((8, n), np.float32)
    rays[0:6] = r6.T
    rays[6] = 0.0
    rays[7] = np.inf
    return rays


def timed(fn, reps=3):
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return out, best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rays", type=int, default=200000)
    args = ap.parse_args()
    if not O.ref_available():
        print(json.dumps({"unavailable": "the reference's sources were not built (oracle/ref/Makefile)"}))
        return 0
    from pbrt_gb300 import scenes as S
    sc = S.displaced_icospheres(seed=3)
    tris = sc["tris"]
    rows = []

    def row(what, port_s, ref_s, units, unit):
        r = {"what": what, "port": round(units / port_s, 4), "reference": round(units / ref_s, 4),
             "unit": unit, "port_over_reference": round(ref_s / port_s, 3)}
        rows.append(r)
        print(json.dumps(r), flush=True)

    port_bvh, tp = timed(lambda: O.BVH(tris), reps=1)
    # the reference's scene set-up (mesh, refinement, primitives) timed
    # without and with its BVHAccel: the difference is the build
    _, tr0 = timed(lambda: O.RefScene(tris, bvh_maxprims=0), reps=1)
    ref_scene, tr = timed(lambda: O.RefScene(tris), reps=1)
    row("SAH BVH build, 1,024,000 triangles", tp, max(tr - tr0, 1e-6), len(tris) / 1e6, "Mtri/s")

    n = args.rays
    sets = {"camera": camera_rays(n), "incoherent": S.random_rays(n, -8.0, 8.0, seed=7)}
    for name, rays in sets.items():
        (a, ta) = timed(lambda: port_bvh.nearest(rays, threads=1))
        (b, tb) = timed(lambda: ref_scene.nearest(rays, use_bvh=True))
        # equal t: a tie between triangles, which each tree breaks by its
        # own visiting order (the intersection kernels take the lower index)
        np.testing.assert_array_equal(a[1], b[1])
        assert np.all((a[0] == b[0]) | (a[1] == b[1]))
        row(f"nearest hit, {name} rays", ta, tb, n / 1e6, "Mrays/s")
        (a, ta) = timed(lambda: port_bvh.anyhit(rays, threads=1))
        (b, tb) = timed(lambda: ref_scene.anyhit(rays, use_bvh=True))
        np.testing.assert_array_equal(a, b)
        row(f"any hit, {name} rays", ta, tb, n / 1e6, "Mrays/s")
    print()
    print(f"{'measurement':44s} {'port':>10s} {'reference':>10s}  unit      port/ref")
    for r in rows:
        print(f"{r['what']:44s} {r['port']:10.3f} {r['reference']:10.3f}  {r['unit']:8s}  {r['port_over_reference']:.2f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
