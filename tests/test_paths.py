"""Every internal path choice gives the same answers: rayhierarchy with and
without triangle clusters (and splitting at any level), ray-bvh with one
thread per ray, persistent warps, warp packets over the ray hierarchy's
leaves or persistent warps over the eight-wide tree (triangle tests per
lane or spread over the warp), the ray image ordered by the direct
Morton permutation (power-of-two sides) or by sorting (other sides), and
host buffers read in place (pageable or pinned) or staged through copies.
All compared bit for bit against the oracle's SAH BVH on the same rays."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def assert_same(got, want, label):
    prim, t, b1, b2 = got
    wprim, wt, _, _ = want
    bad = np.flatnonzero(prim != wprim)
    assert bad.size == 0, f"{label}: {bad.size} prim mismatches, first {bad[:8]}"
    h = prim >= 0
    np.testing.assert_array_equal(t[h].view(np.uint32), wt[h].view(np.uint32), err_msg=label)


@pytest.fixture(scope="module")
def terrain(oracle):
    sc = S.terrain_icospheres(seed=2, grid=96, n_spheres=12)
    tris = sc["tris"]
    cam = S.pinhole_rays(128, 64, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), 50.0, spp=2, jitter_seed=3)
    inc = S.random_rays(12000, [-8, -1, -8], [8, 4, 8], seed=21)
    inc[7, 6000:] = np.random.default_rng(4).uniform(0.1, 4.0, 6000).astype(np.float32)
    B = oracle.BVH(tris)
    return {"tris": tris, "cam": cam, "inc": inc, "B": B,
            "want_cam": B.nearest(cam), "want_inc": B.nearest(inc),
            "occ_inc": B.anyhit(inc)}


@pytest.mark.parametrize("levels", [-1, 1, 2, 4, 99])
def test_rayhierarchy_cluster_levels(gpu_lib, terrain, levels):
    acc = A.MakeAccelerator("rayhierarchy", terrain["tris"], {"clusterLevels": levels})
    assert_same(acc.Intersect(terrain["cam"].copy()), terrain["want_cam"], f"cam, levels {levels}")
    assert_same(acc.Intersect(terrain["inc"].copy()), terrain["want_inc"], f"inc, levels {levels}")
    occ = acc.IntersectP(terrain["inc"])
    np.testing.assert_array_equal(occ == ord("1"), terrain["occ_inc"] == 1)


@pytest.mark.parametrize("walk", [1, 2, 3, 4, 5, 6])
def test_raybvh_walks(gpu_lib, terrain, walk):
    acc = A.MakeAccelerator("ray-bvh", terrain["tris"], {"walk": walk})
    assert_same(acc.Intersect(terrain["cam"].copy()), terrain["want_cam"], f"cam, walk {walk}")
    assert_same(acc.Intersect(terrain["inc"].copy()), terrain["want_inc"], f"inc, walk {walk}")
    occ = acc.IntersectP(terrain["inc"])
    np.testing.assert_array_equal(occ == ord("1"), terrain["occ_inc"] == 1)
    # the bounce form (a validity mask): the incoherent class when automatic
    hit = (np.arange(terrain["inc"].shape[1]) % 3) != 0
    got = acc.Intersect(terrain["inc"].copy(), hit=hit.copy(), bounce=1)
    assert (got[0][~hit] == -1).all()
    np.testing.assert_array_equal(got[0][hit], terrain["want_inc"][0][hit])


@pytest.mark.parametrize("walk", [3, 4, 5, 6])
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_packet_walk_golden(gpu_lib, case, walk):
    """walks 3 and 4 (warp packets over the ray hierarchy's leaves, or over
    the batch in its own order), 5 and 6 (the eight-wide tree, the warp's
    triangle tests on one lane each or spread over its lanes) on the
    reference's own answers: ties, degenerate triangles, limits, empty."""
    g = load_golden(case)
    acc = A.MakeAccelerator("ray-bvh", g["tris"], {"walk": walk})
    got = acc.Intersect(g["rays"].copy())
    np.testing.assert_array_equal(got[0], g["prim"])
    h = g["prim"] >= 0
    np.testing.assert_array_equal(got[1][h], g["t"][h])
    np.testing.assert_array_equal(acc.IntersectP(g["rays"]) == ord("1"), g["occ"] == 1)


def test_packet_walk_sorted_batches(gpu_lib, oracle):
    """walk 3 on batches large enough to be put in the ray hierarchy's
    order (6-D Morton keys; a declared ray image's Morton order), with and
    without a validity mask, nearest and any hit."""
    sc = S.terrain_icospheres(seed=2, grid=96, n_spheres=12)
    tris = sc["tris"]
    B = oracle.BVH(tris)
    acc = A.MakeAccelerator("ray-bvh", tris, {"walk": 3})
    inc = S.random_rays(50000, [-8, -1, -8], [8, 4, 8], seed=31)
    inc[7, ::2] = 2.5
    assert_same(acc.Intersect(inc.copy()), B.nearest(inc), "incoherent")
    np.testing.assert_array_equal(acc.IntersectP(inc) == ord("1"), B.anyhit(inc) == 1)
    hit = (np.arange(inc.shape[1]) % 4) != 1
    got = acc.Intersect(inc.copy(), hit=hit.copy(), bounce=1)
    assert (got[0][~hit] == -1).all()
    np.testing.assert_array_equal(got[0][hit], B.nearest(inc)[0][hit])
    occ = acc.IntersectP(inc, hit=hit.copy())
    np.testing.assert_array_equal(occ[hit] == ord("1"), B.anyhit(inc)[hit] == 1)
    assert (occ[~hit] == ord("0")).all()
    cam = S.pinhole_rays(128, 128, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), 50.0, spp=1, jitter_seed=5)
    acc.Preprocess(None, 1, 1, 1, xres=128, yres=128)
    assert_same(acc.Intersect(cam.copy()), B.nearest(cam), "camera, image order")


@pytest.mark.parametrize("walk", [5, 6])
def test_wide_walk_sorted_masked_and_fallback(gpu_lib, oracle, terrain, walk):
    """walks 5 and 6 over rays in 6-D Morton order, with a validity mask,
    nearest and any hit; and a tree whose leaves exceed the wide format
    (leaves of up to 16 triangles) keeps the two-wide persistent walk with
    the same answers."""
    inc = terrain["inc"]
    acc = A.MakeAccelerator("ray-bvh", terrain["tris"], {"walk": walk, "raySort": 1})
    assert_same(acc.Intersect(inc.copy()), terrain["want_inc"], "sorted")
    hit = (np.arange(inc.shape[1]) % 4) != 1
    got = acc.Intersect(inc.copy(), hit=hit.copy(), bounce=1)
    assert (got[0][~hit] == -1).all()
    np.testing.assert_array_equal(got[0][hit], terrain["want_inc"][0][hit])
    occ = acc.IntersectP(inc, hit=hit.copy())
    np.testing.assert_array_equal(occ[hit] == ord("1"), terrain["occ_inc"][hit] == 1)
    assert (occ[~hit] == ord("0")).all()
    big = A.MakeAccelerator("ray-bvh", terrain["tris"], {"walk": walk, "maxBVHPrim": 16})
    assert_same(big.Intersect(inc.copy()), terrain["want_inc"], "leaves of 16")
    np.testing.assert_array_equal(big.IntersectP(inc) == ord("1"), terrain["occ_inc"] == 1)


def test_wide_tree_device_and_host_collapse(gpu_lib, terrain):
    """The eight-wide tree collapsed on the device (from the device-built
    tree) and on the host (from the host-built tree, the same splits) has
    the same nodes, and walks 5 and 6 over either give the oracle's hits."""
    inc = terrain["inc"]
    stats = []
    for build in (0, 1):
        for walk in (5, 6):
            acc = A.MakeAccelerator("ray-bvh", terrain["tris"], {"bvhBuild": build, "walk": walk})
            assert_same(acc.Intersect(inc.copy()), terrain["want_inc"], f"build {build} walk {walk}")
            np.testing.assert_array_equal(acc.IntersectP(inc) == ord("1"), terrain["occ_inc"] == 1)
            st = acc.stats()
            assert st["wide_nodes"] > 0
            stats.append(st["wide_nodes"])
    assert len(set(stats)) == 1, stats


@pytest.mark.parametrize("width,height", [(128, 64), (96, 80)])
def test_image_order_direct_and_sorted(gpu_lib, oracle, terrain, width, height):
    """A 128 x 64 ray image (power-of-two sides) takes the direct Morton
    permutation, a 96 x 80 one the sort; both give the oracle's hits, with
    and without a validity mask."""
    rays = S.pinhole_rays(width, height, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), 50.0, spp=1,
                          jitter_seed=5)
    want = terrain["B"].nearest(rays)
    acc = A.MakeAccelerator("rayhierarchy", terrain["tris"])
    acc.Preprocess(None, 1, 1, 1, xres=width, yres=height)
    assert_same(acc.Intersect(rays.copy()), want, f"{width}x{height}")
    hit = (np.arange(rays.shape[1]) % 5) != 2
    got = acc.Intersect(rays.copy(), hit=hit.copy(), bounce=1)
    assert (got[0][~hit] == -1).all()
    np.testing.assert_array_equal(got[0][hit], want[0][hit])


def test_host_buffers_pageable_pinned_and_device(gpu_lib, terrain):
    """The host-buffer call on pageable numpy rows, on pinned rows, and the
    device-buffer call give identical results."""
    torch = pytest.importorskip("torch")
    rays = terrain["inc"]
    acc = A.MakeAccelerator("ray-bvh", terrain["tris"])
    pageable = acc.Intersect(rays.copy())
    pinned = torch.empty(rays.shape, dtype=torch.float32, pin_memory=True).numpy()
    pinned[...] = rays
    got_pinned = acc.Intersect(pinned)
    for a, b in zip(pageable, got_pinned):
        np.testing.assert_array_equal(a, b)
    o4 = torch.from_numpy(np.ascontiguousarray(np.stack([rays[0], rays[1], rays[2], rays[6]], 1))).cuda()
    d4 = torch.from_numpy(np.ascontiguousarray(np.stack([rays[3], rays[4], rays[5], rays[7]], 1))).cuda()
    n = rays.shape[1]
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t, b1, b2 = (torch.empty(n, device="cuda") for _ in range(3))
    acc.intersect_device(o4, d4, prim, t, b1, b2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(prim.cpu().numpy(), pageable[0])
    np.testing.assert_array_equal(t.cpu().numpy().view(np.uint32), pageable[1].view(np.uint32))
    assert_same(pageable, terrain["want_inc"], "pageable")


def test_repeated_shadow_origins_reuse_sort(gpu_lib, terrain):
    """Shadow batches from the same points (one per light sample) reuse the
    kept origin order; a batch that moves one origin, changes validity or
    size, or follows a nearest-hit batch, sorts again.  Every batch matches
    the oracle."""
    B = terrain["B"]
    base = terrain["inc"].copy()
    rng = np.random.default_rng(11)
    acc = A.MakeAccelerator("rayhierarchy", terrain["tris"])
    n = base.shape[1]
    all_valid = np.ones(n, bool)
    cases = []
    for k in range(3):  # same origins, new directions and lengths
        r = base.copy()
        r[3:6] = rng.normal(size=(3, n)).astype(np.float32)
        r[7] = rng.uniform(0.5, 6.0, n).astype(np.float32)
        cases.append((r, all_valid))
    other_mint = cases[-1][0].copy()  # the same origins with another mint: no reuse
    other_mint[6] = rng.uniform(0.0, 0.05, n).astype(np.float32)
    cases.append((other_mint, all_valid))
    near = cases[-1][0].copy()  # nearby directions
    near[3:6] += (0.02 * rng.normal(size=(3, n))).astype(np.float32)
    cases.append((near, all_valid))
    cases.append((near, all_valid))  # the same batch again
    moved = cases[-1][0].copy()
    moved[0, n // 2] += 0.75
    cases.append((moved, all_valid))
    some = (np.arange(n) % 7) != 3
    cases.append((moved, some))
    cases.append((moved, some))
    cases.append((moved[:, : n - 64].copy(), some[: n - 64].copy()))
    # per batch: traced in the kept order (reuse), or taken in it and traced
    # again because origins, mint or validity moved (rerun), or sorted afresh
    expect = ["sort", "reuse", "sort", "rerun", "reuse", "reuse", "rerun", "rerun", "reuse", "sort"]
    for i, (r, v) in enumerate(cases):
        if i == 2:  # a nearest-hit batch in between drops the kept order
            assert_same(acc.Intersect(terrain["inc"].copy()), terrain["want_inc"], "nearest")
        before = acc.stats()
        got = acc.IntersectP(r, hit=v) if not v.all() else acc.IntersectP(r)
        after = acc.stats()
        want = B.anyhit(r) == 1
        np.testing.assert_array_equal((got == ord("1"))[v], want[v], err_msg=f"batch {i}")
        seen = (after["origin_reuses"] - before["origin_reuses"], after["origin_reruns"] - before["origin_reruns"])
        assert seen == {"sort": (0, 0), "reuse": (1, 0), "rerun": (0, 1)}[expect[i]], (i, seen)


def test_exact_ties_across_clusters(gpu_lib, oracle):
    """Ties at scale for the front-to-back order with live reach bounds:
    a 48 x 48 grid of quads laid down twice (the second copy after every
    other triangle, so tied triangles sit in different clusters), rays
    straight down onto grid vertices and edge midpoints.  Every ray hits
    several triangles at the same t; the highest index must win, as in the
    in-order loop, although the first cluster reached already set the
    leaf's bound to that t."""
    k = 48
    xs = np.arange(k + 1, dtype=np.float32)
    tris = []
    for i in range(k):
        for j in range(k):
            a = (xs[i], 0.0, xs[j])
            b = (xs[i + 1], 0.0, xs[j])
            c = (xs[i + 1], 0.0, xs[j + 1])
            d = (xs[i], 0.0, xs[j + 1])
            tris.append(a + b + c)
            tris.append(a + c + d)
    tris = np.asarray(tris, np.float32)
    tris = np.concatenate([tris, tris[::-1]])  # each triangle twice, far apart in index
    g = np.random.default_rng(8)
    px = np.concatenate([g.integers(1, k, 6000).astype(np.float32),
                         g.integers(1, k, 3000).astype(np.float32) + 0.5])
    pz = np.concatenate([g.integers(1, k, 6000).astype(np.float32),
                         g.integers(1, k, 3000).astype(np.float32)])
    n = px.size
    rays = np.zeros((8, n), np.float32)
    rays[0], rays[1], rays[2] = px, 3.0, pz
    rays[4] = -1.0
    rays[7] = np.inf
    want = oracle.nearest(tris, rays)
    for kind in ("rayhierarchy", "ray-bvh"):
        acc = A.MakeAccelerator(kind, tris)
        assert_same(acc.Intersect(rays.copy()), want, kind)


@pytest.mark.parametrize("kind", ["rayhierarchy", "ray-bvh"])
def test_host_call_in_two_halves(gpu_lib, kind):
    """A nearest-hit call of 2^21 rays on pinned rows and pinned outputs runs
    as two halves whose copies overlap the other half's traversal; with and
    without a declared ray image and with a validity mask, it answers
    exactly like the device-buffer call."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from pbrt_gb300 import _lib as L
    sc = S.terrain_icospheres(seed=2, grid=96, n_spheres=12)
    rays = S.pinhole_rays(1024, 1024, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), 50.0, spp=2, jitter_seed=9)
    n = rays.shape[1]
    assert n >= 1 << 21
    hit = ((np.arange(n) % 9) != 4).astype(np.uint8)

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    hr = pinned((8, n), torch.float32)
    hr[...] = rays
    hv = pinned((n,), torch.uint8)
    hv[...] = hit
    outs = [pinned((n,), torch.int32)] + [pinned((n,), torch.float32) for _ in range(3)]
    o4 = torch.from_numpy(np.ascontiguousarray(np.stack([rays[0], rays[1], rays[2], rays[6]], 1))).cuda()
    d4 = torch.from_numpy(np.ascontiguousarray(np.stack([rays[3], rays[4], rays[5], rays[7]], 1))).cuda()
    vd = torch.from_numpy(hit).cuda()
    for image in (True, False):
        acc = A.MakeAccelerator(kind, sc["tris"])
        if image:
            acc.Preprocess(None, 2, 1, 1, xres=1024, yres=1024)
        for valid in (None, hv):
            prim = torch.empty(n, dtype=torch.int32, device="cuda")
            t, b1, b2 = (torch.empty(n, device="cuda") for _ in range(3))
            acc.intersect_device(o4, d4, prim, t, b1, b2, valid=None if valid is None else vd)
            torch.cuda.synchronize()
            want = [x.cpu().numpy() for x in (prim, t, b1, b2)]
            h = L.Hits(outs[0].ctypes.data_as(C.POINTER(C.c_int32)),
                       *(o.ctypes.data_as(C.POINTER(C.c_float)) for o in outs[1:]))
            rs = acc._rays_struct(hr, valid)
            L.check(L.lib().pbg_intersect(acc.handle, C.byref(rs), n, C.byref(h)), "pbg_intersect")
            for a, b in zip(outs, want):
                np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("kind", ["rayhierarchy", "ray-bvh"])
def test_host_shadow_call_in_two_parts(gpu_lib, kind):
    """A shadow call of 2^21 rays on pinned rows and a pinned result runs as
    two parts with their own work buffers and kept origin orders; through
    repeated light samples (both parts reuse their order), a validity change
    in the second part only, a nearest-hit call in between and a call
    without a mask, it answers exactly like the device-buffer call of a
    separate accelerator."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from pbrt_gb300 import _lib as L
    sc = S.terrain_icospheres(seed=3, grid=96, n_spheres=12)
    cam = S.pinhole_rays(1024, 1024, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), 50.0, spp=2, jitter_seed=4)
    n = cam.shape[1]
    assert n >= 1 << 21
    acc = A.MakeAccelerator(kind, sc["tris"])
    ref = A.MakeAccelerator(kind, sc["tris"])
    prim, t, _, _ = acc.Intersect(cam.copy())
    hitm = prim >= 0
    p = cam[0:3] + cam[3:6] * np.where(hitm, t, 0)[None]
    rng = np.random.default_rng(5)

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    def shadow(q):
        lp = np.array([[0.6 * q - 1.0], [8.5], [0.3 * q]], np.float32) + rng.uniform(-0.2, 0.2, (3, n)).astype(np.float32)
        d = lp - p
        out = np.empty((8, n), np.float32)
        out[0:3] = p
        out[3:6] = d
        out[6] = 1e-3
        out[7] = 0.999
        return out

    hr = pinned((8, n), torch.float32)
    hv = pinned((n,), torch.uint8)
    ho = pinned((n,), torch.uint8)
    mask = hitm.astype(np.uint8)
    moved = mask.copy()
    moved[n - 1000:n - 990] ^= 1  # second part only
    steps = [(0, mask), (1, mask), (2, mask), (2, moved), ("cam", None), (3, mask), (3, None)]
    reuses = acc.stats()["origin_reuses"]
    for q, m in steps:
        if q == "cam":
            acc.Intersect(cam.copy())
            continue
        hr[...] = shadow(q)
        if m is not None:
            hv[...] = m
        rs = acc._rays_struct(hr, None if m is None else hv)
        L.check(L.lib().pbg_occluded(acc.handle, C.byref(rs), n, ho.ctypes.data), "pbg_occluded")
        o4 = torch.from_numpy(np.ascontiguousarray(np.stack([hr[0], hr[1], hr[2], hr[6]], 1))).cuda()
        d4 = torch.from_numpy(np.ascontiguousarray(np.stack([hr[3], hr[4], hr[5], hr[7]], 1))).cuda()
        occ = torch.empty(n, dtype=torch.uint8, device="cuda")
        ref.occluded_device(o4, d4, occ, valid=None if m is None else torch.from_numpy(m).cuda())
        torch.cuda.synchronize()
        want = occ.cpu().numpy()
        np.testing.assert_array_equal(ho != 0, want != 0, err_msg=f"{kind} step {q}")
        assert 0 < int(np.count_nonzero(want)) < n
    if kind == "rayhierarchy":  # light samples 1 and 2 in both parts, 2 with the moved mask in part one
        assert acc.stats()["origin_reuses"] - reuses == 5
    # a size that is no multiple of 4,096: the part boundary is rounded down
    # to one, and the second part ends on a ragged tail
    extra = 3001
    rows = np.concatenate([shadow(4), shadow(5)[:, :extra]], 1)
    m2 = np.concatenate([mask, mask[:extra]])
    n2 = rows.shape[1]
    hr2 = pinned((8, n2), torch.float32)
    hr2[...] = rows
    hv2 = pinned((n2,), torch.uint8)
    hv2[...] = m2
    ho2 = pinned((n2,), torch.uint8)
    rs = acc._rays_struct(hr2, hv2)
    L.check(L.lib().pbg_occluded(acc.handle, C.byref(rs), n2, ho2.ctypes.data), "pbg_occluded")
    o4 = torch.from_numpy(np.ascontiguousarray(np.stack([rows[0], rows[1], rows[2], rows[6]], 1))).cuda()
    d4 = torch.from_numpy(np.ascontiguousarray(np.stack([rows[3], rows[4], rows[5], rows[7]], 1))).cuda()
    occ = torch.empty(n2, dtype=torch.uint8, device="cuda")
    ref.occluded_device(o4, d4, occ, valid=torch.from_numpy(m2).cuda())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ho2 != 0, occ.cpu().numpy() != 0, err_msg=f"{kind} ragged size")


@pytest.mark.parametrize("seed", range(6))
def test_randomised_scenes_against_oracle(gpu_lib, oracle, seed):
    """Randomised scenes (terrain with icospheres at random sizes, a grid of
    shared-edge quads laid over it, a random soup) and ray sets (a declared
    camera image with jitter, masked shadow batches from its hits reused
    across light samples, incoherent segments): rayhierarchy and ray-bvh
    against the oracle, bit for bit."""
    rng = np.random.default_rng(100 + seed)
    sc = S.terrain_icospheres(seed=seed, grid=int(rng.integers(32, 96)), n_spheres=int(rng.integers(2, 20)))
    k = 24
    xs = np.linspace(-4, 4, k + 1, dtype=np.float32)
    quads = []
    for i in range(k):
        for j in range(k):
            a = (xs[i], 1.5, xs[j]); b = (xs[i + 1], 1.5, xs[j]); c = (xs[i + 1], 1.5, xs[j + 1]); d = (xs[i], 1.5, xs[j + 1])
            quads.append(a + b + c)
            quads.append(a + c + d)
    soup = rng.uniform(-6, 6, (500, 9)).astype(np.float32)
    soup[:, 3:] = soup[:, :3].repeat(2, 0).reshape(-1, 6) + rng.normal(0, 0.3, (500, 6)).astype(np.float32)
    tris = np.concatenate([sc["tris"], np.asarray(quads, np.float32), soup])
    tris = tris[rng.permutation(len(tris))]
    B = oracle.BVH(tris)
    w, h = 128, 64
    cam = S.pinhole_rays(w, h, tuple(rng.uniform([-3, 5, -12], [3, 10, -8])), (0.0, 0.0, 0.0),
                         float(rng.uniform(30, 70)), spp=2, jitter_seed=seed)
    inc = S.random_rays(8000, [-8, -1, -8], [8, 5, 8], seed=seed)
    inc[7, ::2] = rng.uniform(0.05, 6.0, 4000).astype(np.float32)
    for kind in ("rayhierarchy", "ray-bvh"):
        acc = A.MakeAccelerator(kind, tris)
        acc.Preprocess(None, 2, 1, 1, xres=w, yres=h)
        want = B.nearest(cam)
        assert_same(acc.Intersect(cam.copy()), want, f"{kind} camera {seed}")
        hitm = want[0] >= 0
        p = cam[0:3] + cam[3:6] * np.where(hitm, want[1], 0)[None]
        for q in range(3):
            lp = rng.uniform([-1, 8, -1], [1, 9, 1], (cam.shape[1], 3)).T
            d = lp - p
            dist = np.sqrt((d ** 2).sum(0))
            dist = np.where(dist > 0, dist, 1.0)
            r = np.empty((8, cam.shape[1]), np.float32)
            r[0:3] = p
            r[3:6] = d / dist[None]
            r[6] = np.where(hitm, 1e-3 * want[1], 0.0)
            r[7] = dist * (1 - 1e-3)
            occ = acc.IntersectP(r, hit=hitm)
            want_occ = B.anyhit(r, valid=hitm.astype(np.uint8)) == 1
            np.testing.assert_array_equal((occ == ord("1"))[hitm], want_occ[hitm], err_msg=f"{kind} shadow {seed}/{q}")
        assert_same(acc.Intersect(inc.copy()), B.nearest(inc), f"{kind} incoherent {seed}")
        np.testing.assert_array_equal(acc.IntersectP(inc) == ord("1"), B.anyhit(inc) == 1)


def test_device_entry_reruns_on_a_caller_stream(gpu_lib, oracle):
    """The device entry points on a caller's stream, through the two paths
    that trace a batch again after its first attempt already wrote the
    caller's arrays: a pair-queue overflow (a million incoherent rays of
    unbounded length against the 181,250-triangle scene with its pair
    queues held to 2^18 pairs, the scene's first call) and a shadow batch
    whose origins moved from the kept order.  The final results equal the
    oracle's."""
    import torch
    sc = S.terrain_icospheres(seed=2)
    tris = sc["tris"]
    acc = A.MakeAccelerator("rayhierarchy", tris, {"queuePairs": 1 << 18})
    B = oracle.BVH(tris)
    stream = torch.cuda.Stream()
    rays = S.random_rays(1 << 20, [-8, -1, -8], [8, 4, 8], seed=41)

    def dev(r):
        o = torch.from_numpy(np.ascontiguousarray(np.stack([r[0], r[1], r[2], r[6]], 1))).cuda()
        d = torch.from_numpy(np.ascontiguousarray(np.stack([r[3], r[4], r[5], r[7]], 1))).cuda()
        return o, d

    n = rays.shape[1]
    o4, d4 = dev(rays)
    prim = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    t, b1, b2 = (torch.full((n,), 7.0, device="cuda") for _ in range(3))
    before = acc.stats()
    with torch.cuda.stream(stream):
        acc.intersect_device(o4, d4, prim, t, b1, b2, stream=stream)
    stream.synchronize()
    assert acc.stats()["queue_reruns"] > before["queue_reruns"]
    want = B.nearest(rays)
    assert_same([x.cpu().numpy() for x in (prim, t, b1, b2)], want, "overflow rerun")
    # shadow batches: the same origins twice (kept order), then one moved
    base = rays[:, :200000].copy()
    g = np.random.default_rng(5)
    cases = []
    for k in range(2):
        r = base.copy()
        r[3:6] = g.normal(size=(3, r.shape[1])).astype(np.float32)
        r[7] = g.uniform(0.5, 6.0, r.shape[1]).astype(np.float32)
        cases.append(r)
    moved = cases[-1].copy()
    moved[0, 1000] += 0.5
    cases.append(moved)
    occ = torch.full((base.shape[1],), 9, dtype=torch.uint8, device="cuda")
    for i, r in enumerate(cases):
        so, sd = dev(r)
        before = acc.stats()
        with torch.cuda.stream(stream):
            acc.occluded_device(so, sd, occ, stream=stream)
        stream.synchronize()
        after = acc.stats()
        if i == 2:
            assert after["origin_reruns"] == before["origin_reruns"] + 1
        np.testing.assert_array_equal(occ.cpu().numpy(), B.anyhit(r), err_msg=f"shadow batch {i}")
