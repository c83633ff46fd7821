"""Generates the golden fixtures in this directory from the reference's own
CPU code (oracle/_ref/libpbrtref.so, built by oracle/ref/Makefile from the
pbrt-v2 fork's sources: Triangle::Intersect/IntersectP, GeometricPrimitive,
BVHAccel, DifferentialGeometry).

Run in a checkout that has the reference tree next to it:
    python tests/golden/make_golden.py
Each case is one .npz holding its inputs (triangles, rays, uvs) and the
reference's answers:
    prim/t/b1/b2   nearest hit, primitives tested in index order with pbrt's
                   maxt update (the semantics of a sequential aggregate)
    bvh_prim/...   the same through pbrt's BVHAccel (differs only on exact
                   ties in t, which the in-order loop resolves to the highest
                   index)
    occ            shadow any-hit through IntersectP
    geo            [n, 14] DifferentialGeometry (p, dpdu, dpdv, nn, u, v) from
                   a second scene built with the case's uv mode
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import pbg_import  # noqa: E402

pbg_import.load()
from pbrt_gb300 import scenes as S  # noqa: E402

F32 = np.float32


def grid_scene(n=8, size=1.0):
    """n x n unit quads in the plane z = 0, two triangles each."""
    tris = []
    for i in range(n):
        for j in range(n):
            a = (i * size, j * size, 0.0)
            b = ((i + 1) * size, j * size, 0.0)
            c = ((i + 1) * size, (j + 1) * size, 0.0)
            d = (i * size, (j + 1) * size, 0.0)
            tris.append(a + b + c)
            tris.append(a + c + d)
    return np.array(tris, F32)


def rays_from(o, d, mint=0.0, maxt=np.inf):
    o = np.asarray(o, np.float64)
    d = np.asarray(d, np.float64)
    n = max(len(o), len(d))
    r = np.empty((8, n), F32)
    r[0:3] = np.broadcast_to(o, (n, 3)).T
    r[3:6] = np.broadcast_to(d, (n, 3)).T
    r[6] = mint
    r[7] = maxt
    return r


def case_grid_ties(rng):
    tris = grid_scene(8)
    pts = []
    # lattice vertices, edge midpoints, cell centres: exact ties on shared edges
    for x in np.arange(0, 8.01, 0.5):
        for y in np.arange(0, 8.01, 0.5):
            pts.append((x, y))
    pts = np.array(pts)
    o = np.c_[pts, np.full(len(pts), 3.0)]
    down = rays_from(o, (0.0, 0.0, -1.0))
    # slanted rays aimed at the same lattice points
    d = np.c_[rng.uniform(-0.3, 0.3, (len(pts), 2)), -np.ones(len(pts))]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o2 = np.c_[pts, np.zeros(len(pts))] - 4.0 * d
    slant = rays_from(o2, d)
    # rays lying in the plane, parallel to it, with zero direction components
    flat = rays_from(np.c_[rng.uniform(-1, 9, (64, 2)), np.zeros(64)],
                     np.c_[rng.normal(size=(64, 2)), np.zeros(64)])
    par = rays_from(np.c_[rng.uniform(-1, 9, (64, 2)), np.full(64, 0.25)],
                    np.c_[rng.normal(size=(64, 2)), np.zeros(64)])
    rays = np.concatenate([down, slant, flat, par], 1)
    rays[3:6] /= np.linalg.norm(rays[3:6].astype(np.float64), axis=0).astype(F32)
    return tris, rays


def case_degenerate(rng):
    good = rng.uniform(-2, 2, (40, 9)).astype(F32)
    rep = good.copy()[:20]
    rep[:, 6:9] = rep[:, 3:6]                     # p3 == p2
    col = good.copy()[:20]
    col[:, 6:9] = 0.5 * (col[:, 0:3] + col[:, 3:6])  # collinear
    tiny = good[:10].copy()
    tiny[:, 3:9] = tiny[:, 0:3][:, [0, 1, 2, 0, 1, 2]] + rng.uniform(-1e-6, 1e-6, (10, 6))
    huge = (good[:10] * 1e4).astype(F32)
    tris = np.concatenate([good, rep, col, tiny, huge], 0).astype(F32)
    rays = S.random_rays(1500, -3.0, 3.0, seed=int(rng.integers(1 << 30)))
    # rays aimed at vertices and edge midpoints of the good triangles
    tgt = np.concatenate([good[:, 0:3], 0.5 * (good[:, 0:3] + good[:, 3:6])], 0)
    src = rng.uniform(-6, 6, (len(tgt), 3))
    d = tgt - src
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([rays, rays_from(src, d)], 1)
    return tris, rays


def case_soup(rng):
    c = rng.uniform(-5, 5, (600, 3))
    tris = (np.repeat(c, 3, axis=0) + rng.normal(scale=0.6, size=(1800, 3))).reshape(600, 9)
    tris = tris.astype(F32)
    rays = S.random_rays(3000, -6.0, 6.0, seed=int(rng.integers(1 << 30)))
    # segments: finite maxt, mint > 0
    rays[6, 1000:2000] = rng.uniform(0.0, 0.5, 1000)
    rays[7, 1000:2000] = rng.uniform(0.5, 6.0, 1000)
    uvs = rng.uniform(-1, 2, (600, 6)).astype(F32)
    uvs[::7, 4:6] = uvs[::7, 0:2]  # zero uv determinant: CoordinateSystem fallback
    return tris, rays, uvs


def case_sphere_small():
    cfg = S.config_small_naive()
    rays = cfg["rays"][:, ::16].copy()
    return cfg["tris"], rays, cfg["light"]


def shadow_from_hits(rays, prim, t, light):
    hit = prim >= 0
    p = rays[0:3, hit] + rays[3:6, hit] * t[hit][None]
    return S.shadow_rays_to_point(p.T.astype(F32), light)


def ref_answers(tris, rays, uv_mode_geo=0, uvs=None, with_geo=True):
    R = O.RefScene(tris, uv_mode=1)
    prim, t, b1, b2 = R.nearest(rays, use_bvh=False)
    bprim, bt, bb1, bb2 = R.nearest(rays, use_bvh=True)
    occ = R.anyhit(rays, use_bvh=False)
    out = dict(tris=tris, rays=rays, prim=prim, t=t, b1=b1, b2=b2, bvh_prim=bprim, bvh_t=bt,
               occ=occ)
    if with_geo:
        G = O.RefScene(tris, uv_mode=uv_mode_geo, uvs=uvs)
        gp, gt, gu, gv, geo = G.nearest(rays, use_bvh=False, geometry=True)
        assert np.array_equal(gp, prim) and np.array_equal(gt, t)
        out["geo"] = geo
        out["geo_uv_mode"] = np.int32(uv_mode_geo)
        if uvs is not None:
            out["uvs"] = uvs
    return out


SMALL_CAMERA = dict(eye=(0.0, 1.0, -4.0), look=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov=45.0)
SMALL_LIGHT = dict(pos=(2.0, 4.0, -2.0), I=(16.0, 16.0, 16.0))


def small_scene_text(tris, out_name="out.pfm"):
    """The small naive workload as a pbrt scene file: 256x256, 1 spp at pixel
    centres, point light, matte 0.7, directlighting, the CPU "bvh"."""
    n = len(tris)
    P = " ".join(repr(float(x)) for x in tris.reshape(-1))
    idx = " ".join(str(i) for i in range(3 * n))
    c, l = SMALL_CAMERA, SMALL_LIGHT
    return f'''LookAt {c["eye"][0]} {c["eye"][1]} {c["eye"][2]}  {c["look"][0]} {c["look"][1]} {c["look"][2]}  {c["up"][0]} {c["up"][1]} {c["up"][2]}
Camera "perspective" "float fov" [{c["fov"]}]
Sampler "stratified" "integer xsamples" [1] "integer ysamples" [1] "bool jitter" ["false"]
PixelFilter "box"
Film "image" "integer xresolution" [256] "integer yresolution" [256] "string filename" ["{out_name}"]
Renderer "sampler"
SurfaceIntegrator "directlighting"
Accelerator "bvh"
WorldBegin
LightSource "point" "point from" [{l["pos"][0]} {l["pos"][1]} {l["pos"][2]}] "rgb I" [{l["I"][0]} {l["I"][1]} {l["I"][2]}]
Material "matte" "rgb Kd" [0.7 0.7 0.7]
Shape "trianglemesh" "integer indices" [{idx}] "point P" [{P}]
WorldEnd
'''


def case_render_small():
    import tempfile
    cfg = S.config_small_naive()
    tris = cfg["tris"]
    xs, ys = np.meshgrid(np.arange(256), np.arange(256))
    xy = np.stack([xs.reshape(-1) + 0.5, ys.reshape(-1) + 0.5], 1).astype(np.float32)
    c = SMALL_CAMERA
    r2c, c2w, rays6 = O.ref_camera(256, 256, c["eye"], c["look"], c["up"], c["fov"], xy)
    with tempfile.TemporaryDirectory() as td:
        img = O.ref_render(small_scene_text(tris), td)
    sel = np.arange(0, len(xy), 7)
    return dict(r2c=r2c, c2w=c2w, image=img, camera_xy=xy[sel], camera_rays=rays6[sel],
                light_pos=np.array(SMALL_LIGHT["pos"], np.float32),
                light_I=np.array(SMALL_LIGHT["I"], np.float32),
                albedo=np.array([0.7, 0.7, 0.7], np.float32))


# The breadth-first renders (Renderer "breadth-first", Accelerator "naive"
# through the CPU batch backend of oracle/ref): the small sphere workload
# plus a 2-triangle area light that the camera sees.
BF = dict(xres=48, yres=40, spp=(2, 2), eye=(0.0, 0.3, -4.5), look=(0.0, 1.3, 0.0), up=(0.0, 1.0, 0.0),
          fov=55.0, L=(5.0, 5.0, 5.0), nsamples=4, max_depth=5)
BF_QUAD = np.array([[-1, 3, -1], [1, 3, -1], [1, 3, 1], [-1, 3, 1]], F32)


def bf_scene_text(tris, integrator, light_text, out_name="out.pfm"):
    n = len(tris)
    P = " ".join(repr(float(x)) for x in tris.reshape(-1))
    idx = " ".join(str(i) for i in range(3 * n))
    c = BF
    extra = f' "integer maxdepth" [{c["max_depth"]}]' if integrator == "path" else ""
    return f'''LookAt {c["eye"][0]} {c["eye"][1]} {c["eye"][2]}  {c["look"][0]} {c["look"][1]} {c["look"][2]}  {c["up"][0]} {c["up"][1]} {c["up"][2]}
Camera "perspective" "float fov" [{c["fov"]}]
Sampler "stratified" "integer xsamples" [{c["spp"][0]}] "integer ysamples" [{c["spp"][1]}] "bool jitter" ["true"]
PixelFilter "box"
Film "image" "integer xresolution" [{c["xres"]}] "integer yresolution" [{c["yres"]}] "string filename" ["{out_name}"]
Renderer "breadth-first"
SurfaceIntegrator "{integrator}"{extra}
Accelerator "naive"
WorldBegin
Material "matte" "rgb Kd" [0.7 0.7 0.7]
Shape "trianglemesh" "integer indices" [{idx}] "point P" [{P}]
{light_text}WorldEnd
'''


def case_render_bf():
    import tempfile
    from pbrt_gb300 import render as R
    base = S.config_small_naive()["tris"]
    c = BF
    Q = " ".join(repr(float(x)) for x in BF_QUAD.reshape(-1))
    area = (f'AttributeBegin\nAreaLightSource "diffuse" "rgb L" [{c["L"][0]} {c["L"][1]} {c["L"][2]}] '
            f'"integer nsamples" [{{ns}}]\nShape "trianglemesh" "integer indices" [0 1 2 0 2 3] "point P" [{Q}]\n'
            'AttributeEnd\n')
    point = 'LightSource "point" "point from" [0 3 0] "rgb I" [8 8 8]\n'
    out = {}
    with tempfile.TemporaryDirectory() as td:
        out["image_direct"] = O.ref_render(bf_scene_text(base, "directlighting", area.format(ns=c["nsamples"])), td)
        out["image_path"] = O.ref_render(bf_scene_text(base, "path", area.format(ns=1)), td)
        out["image_point"] = O.ref_render(bf_scene_text(base, "directlighting", point), td)
    r2c, c2w, _ = O.ref_camera(c["xres"], c["yres"], c["eye"], c["look"], c["up"], c["fov"],
                               np.zeros((1, 2), F32))
    out.update(r2c=r2c, c2w=c2w, quad=BF_QUAD)
    # pins of the restated sampler: pbrt's own first samples and RNG draws
    ext = (0, c["xres"] + 1, 0, c["yres"] + 1)
    for tag, integ, nsl in (("path", "path", [1]), ("direct", "directlighting", [c["nsamples"]])):
        n1d, n2d = R.sample_arrays(integ, nsl)
        img, o1, o2, rng = O.pbrt_task_samples(ext, c["spp"], n1d, n2d, 64, 2048, reference=True)
        out.update({f"samp_{tag}_img": img, f"samp_{tag}_oned": o1, f"samp_{tag}_twod": o2, f"samp_{tag}_rng": rng})
    # pins of the restated area light: pbrt's DiffuseAreaLight::Sample_L
    g = np.random.default_rng(11)
    quad_tris = np.array([np.r_[BF_QUAD[0], BF_QUAD[1], BF_QUAD[2]], np.r_[BF_QUAD[0], BF_QUAD[2], BF_QUAD[3]]], F32)
    uneven = g.uniform(-1, 1, (7, 9)).astype(F32)
    uneven[:, 1::3] += 3.0
    for tag, lt in (("quad", quad_tris), ("uneven", uneven)):
        q = np.zeros((256, 7), F32)
        q[:, 0:3] = g.uniform([-3, -1, -3], [3, 2.9, 3], (256, 3))
        q[:, 3] = 1e-3
        q[:, 4:7] = g.random((256, 3))
        out.update({f"light_{tag}_tris": lt, f"light_{tag}_q": q,
                    f"light_{tag}_out": O.area_light_sample(lt, c["L"], q, reference=True)})
    return out


def main():
    if not O.ref_available():
        if not O.build_ref():
            sys.exit("reference tree not found: cannot build oracle/_ref")
    O.build()
    rng = np.random.default_rng(20261203)

    tris, rays, light = case_sphere_small()
    a = ref_answers(tris, rays)
    sh = shadow_from_hits(rays, a["prim"], a["t"], light)
    R = O.RefScene(tris, uv_mode=1)
    a["shadow_rays"] = sh
    a["shadow_occ"] = R.anyhit(sh)
    a["shadow_occ_bvh"] = R.anyhit(sh, use_bvh=True)
    np.savez_compressed(os.path.join(HERE, "sphere_small.npz"), **a)

    tris, rays = case_grid_ties(rng)
    np.savez_compressed(os.path.join(HERE, "grid_ties.npz"), **ref_answers(tris, rays))

    tris, rays = case_degenerate(rng)
    np.savez_compressed(os.path.join(HERE, "degenerate.npz"), **ref_answers(tris, rays))

    tris, rays, uvs = case_soup(rng)
    np.savez_compressed(os.path.join(HERE, "soup.npz"),
                        **ref_answers(tris, rays, uv_mode_geo=2, uvs=uvs))

    # t == maxt is accepted, t == mint is accepted (shapes/trianglemesh.cpp:152)
    tris = grid_scene(2)
    o = np.array([[0.25, 0.25, 2.0], [1.5, 0.75, 3.0], [0.6, 1.7, 1.0]])
    base = rays_from(o, (0.0, 0.0, -1.0))
    R = O.RefScene(tris, uv_mode=1)
    p0, t0, _, _ = R.nearest(base)
    eq_max = base.copy()
    eq_max[7] = t0
    eq_min = base.copy()
    eq_min[6] = t0
    below = base.copy()
    below[7] = np.nextafter(t0, np.float32(0))
    above = base.copy()
    above[6] = np.nextafter(t0, np.float32(np.inf))
    rays = np.concatenate([eq_max, eq_min, below, above], 1)
    np.savez_compressed(os.path.join(HERE, "limits.npz"), **ref_answers(tris, rays))

    # the reference's own render of the small naive workload
    np.savez_compressed(os.path.join(HERE, "render_small.npz"), **case_render_small())

    # the reference's breadth-first renders with an area light
    np.savez_compressed(os.path.join(HERE, "render_bf.npz"), **case_render_bf())

    # empty scene
    tris = np.zeros((0, 9), F32)
    rays = S.random_rays(16, -1.0, 1.0, seed=5)
    np.savez_compressed(os.path.join(HERE, "empty.npz"), tris=tris, rays=rays,
                        prim=np.full(16, -1, np.int32), t=np.zeros(16, F32),
                        b1=np.zeros(16, F32), b2=np.zeros(16, F32), occ=np.zeros(16, np.uint8))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
