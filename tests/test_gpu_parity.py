"""GPU parity: every accelerator, through the C ABI, against the oracle and
the reference's golden answers.  The bar is bit-exact prim/t/b1/b2 and
occlusion (the tie rule of the in-order loop is part of the contract)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

pytestmark = pytest.mark.gpu

KINDS = ["naive", "ray-bvh", "rayhierarchy"]


def make(kind, tris, uvs=None, ps=None):
    return A.MakeAccelerator(kind, tris, ps, uvs)


def assert_hits_equal(got, want, label=""):
    prim, t, b1, b2 = got
    wprim, wt, wb1, wb2 = want
    bad = np.flatnonzero(prim != wprim)
    assert bad.size == 0, f"{label}: {bad.size} prim mismatches, first {bad[:8]} got {prim[bad[:8]]} want {wprim[bad[:8]]}"
    h = prim >= 0
    np.testing.assert_array_equal(t[h].view(np.uint32), wt[h].view(np.uint32), err_msg=label)
    np.testing.assert_array_equal(b1[h], wb1[h], err_msg=label)
    np.testing.assert_array_equal(b2[h], wb2[h], err_msg=label)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_nearest(gpu_lib, kind, case):
    g = load_golden(case)
    acc = make(kind, g["tris"])
    rays = g["rays"].copy()
    got = acc.Intersect(rays)
    assert_hits_equal(got, (g["prim"], g["t"], g["b1"], g["b2"]), f"{kind}/{case}")
    # the reference sets r.maxt = t on every hit
    h = got[0] >= 0
    np.testing.assert_array_equal(rays[7, h], g["t"][h])


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_occluded(gpu_lib, kind, case):
    g = load_golden(case)
    acc = make(kind, g["tris"])
    occ = acc.IntersectP(g["rays"])
    np.testing.assert_array_equal(occ == ord("1"), g["occ"] == 1)


@pytest.mark.parametrize("kind", KINDS)
def test_golden_shadow_rays(gpu_lib, kind):
    g = load_golden("sphere_small")
    acc = make(kind, g["tris"])
    occ = acc.IntersectP(g["shadow_rays"])
    np.testing.assert_array_equal(occ == ord("1"), g["shadow_occ"] == 1)


@pytest.mark.parametrize("case", ["sphere_small", "soup"])
def test_golden_hit_geometry(gpu_lib, case):
    g = load_golden(case)
    uvs = g.get("uvs")
    acc = make("naive", g["tris"], uvs=uvs)
    geo = acc.HitGeometry(g["rays"], g["prim"], g["t"], g["b1"], g["b2"])
    np.testing.assert_array_equal(geo, g["geo"])


@pytest.mark.parametrize("kind", KINDS)
def test_small_config_against_oracle(gpu_lib, oracle, kind):
    """The full 256x256 naive workload (4,034 triangles, 65,536 camera rays)
    plus its shadow rays, against the oracle."""
    cfg = S.config_small_naive()
    tris, rays = cfg["tris"], cfg["rays"]
    want = oracle.nearest(tris, rays)
    acc = make(kind, tris)
    got = acc.Intersect(rays.copy())
    assert_hits_equal(got, want, kind)
    hit = want[0] >= 0
    p = rays[0:3, hit] + rays[3:6, hit] * want[1][hit][None]
    sh = S.shadow_rays_to_point(p.T.astype(np.float32), cfg["light"])
    np.testing.assert_array_equal(acc.IntersectP(sh) == ord("1"), oracle.anyhit(tris, sh) == 1)


@pytest.mark.parametrize("kind", KINDS)
def test_incoherent_rays_terrain(gpu_lib, oracle, kind):
    """Incoherent segments in the terrain + icospheres scene (181,250
    triangles); the oracle's BVH port answers like the in-order loop."""
    sc = S.terrain_icospheres(seed=2)
    tris = sc["tris"]
    rays = S.random_rays(20000, [-8, -1, -8], [8, 4, 8], seed=11)
    rays[7, 10000:] = np.random.default_rng(3).uniform(0.1, 5.0, 10000).astype(np.float32)
    B = oracle.BVH(tris)
    want = B.nearest(rays)
    acc = make(kind, tris)
    got = acc.Intersect(rays.copy())
    assert_hits_equal(got, want, kind)
    np.testing.assert_array_equal(acc.IntersectP(rays) == ord("1"), B.anyhit(rays) == 1)


@pytest.mark.parametrize("kind", KINDS)
def test_bounce_mask_and_invalid_rays(gpu_lib, oracle, kind):
    g = load_golden("soup")
    acc = make(kind, g["tris"])
    n = g["rays"].shape[1]
    hit = (np.arange(n) % 4 != 1)
    hit_io = hit.copy()
    prim, t, b1, b2 = acc.Intersect(g["rays"].copy(), hit=hit_io, bounce=1)
    assert (prim[~hit] == -1).all()
    np.testing.assert_array_equal(prim[hit], g["prim"][hit])
    np.testing.assert_array_equal(hit_io, hit & (g["prim"] >= 0))
    occ = acc.IntersectP(g["rays"], hit=hit)
    assert (occ[~hit] == ord("0")).all()
    np.testing.assert_array_equal(occ[hit] == ord("1"), g["occ"][hit] == 1)


def test_accelerators_agree_at_scale(gpu_lib):
    """Size-independent property at the full ray-hierarchy workload size:
    the three accelerators return identical hits for 4.19M camera rays
    (1024x1024, 4 spp jittered) on 181,250 triangles; naive is the exact
    all-pairs loop."""
    sc = S.terrain_icospheres(seed=2)
    tris = sc["tris"]
    rays = S.pinhole_rays(1024, 1024, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), 50.0, spp=4,
                          jitter_seed=7)
    sub = rays[:, ::8].copy()  # 524,288 rays keeps the all-pairs run short
    ref = make("naive", tris).Intersect(sub.copy())
    for kind in ("ray-bvh", "rayhierarchy"):
        got = make(kind, tris).Intersect(sub.copy())
        assert_hits_equal(got, ref, kind)


@pytest.mark.parametrize("kind", KINDS)
def test_ray_image_layout(gpu_lib, oracle, kind):
    """Preprocess declares the breadth-first ray image (256 x 256, 1 spp);
    the ray hierarchy then groups rays by 2-D image tiles.  Shadow batches
    keep the layout with a validity mask."""
    cfg = S.config_small_naive()
    tris, rays = cfg["tris"], cfg["rays"]
    acc = make(kind, tris)
    acc.Preprocess(None, 1, 1, 1, xres=256, yres=256)
    want = oracle.nearest(tris, rays)
    got = acc.Intersect(rays.copy())
    assert_hits_equal(got, want, kind)
    hit = want[0] >= 0
    p = rays[0:3] + rays[3:6] * np.where(hit, want[1], 0)[None]
    sh = S.shadow_rays_to_point(p.T.astype(np.float32), cfg["light"])
    occ = acc.IntersectP(sh, hit=hit)
    np.testing.assert_array_equal(occ == ord("1"), oracle.anyhit(tris, sh, valid=hit.astype(np.uint8)) == 1)
