"""pbg_autotune: every launch shape it tries answers identically (the call
checks that bit for bit and reports the mismatch count), and the scene's
answers after tuning equal the oracle's, for nearest-hit and any-hit
batches on every accelerator."""
import numpy as np
import pytest

from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

pytestmark = pytest.mark.gpu

EXPECTED = {"naive": 4, "rayhierarchy": 6, "ray-bvh": 6}


def dev(rays):
    import torch
    o = torch.from_numpy(np.ascontiguousarray(np.stack([rays[0], rays[1], rays[2], rays[6]], 1))).cuda()
    d = torch.from_numpy(np.ascontiguousarray(np.stack([rays[3], rays[4], rays[5], rays[7]], 1))).cuda()
    return o, d


@pytest.mark.parametrize("kind", ["naive", "rayhierarchy", "ray-bvh"])
def test_tuned_shapes_answer_identically(gpu_lib, oracle, kind):
    import torch
    sc = S.terrain_icospheres(seed=2, grid=48, n_spheres=6)
    tris = sc["tris"]
    rays = S.random_rays(1 << 17 if kind != "naive" else 1 << 14, [-8, -1, -8], [8, 4, 8], seed=23)
    rays[7, ::3] = 4.0
    acc = A.MakeAccelerator(kind, tris)
    o4, d4 = dev(rays)
    for anyhit, incoherent in ((False, False), (True, False), (False, True)):
        r = acc.autotune(o4, d4, anyhit=anyhit, incoherent=incoherent, reps=2)
        assert r["mismatches"] == 0
        assert len(r["candidates"]) == EXPECTED[kind]
        assert r["best"] in [c["setting"] for c in r["candidates"]]
        assert all(c["ms"] > 0 for c in r["candidates"])
    B = oracle.BVH(tris)
    want = B.nearest(rays)
    n = rays.shape[1]
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t, b1, b2 = (torch.empty(n, device="cuda") for _ in range(3))
    acc.intersect_device(o4, d4, prim, t, b1, b2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(prim.cpu().numpy(), want[0])
    h = want[0] >= 0
    np.testing.assert_array_equal(t.cpu().numpy()[h], want[1][h])
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    acc.occluded_device(o4, d4, occ)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(occ.cpu().numpy(), B.anyhit(rays))
    acc.close()


def test_fixed_walk_is_not_tuned(gpu_lib):
    sc = S.terrain_icospheres(seed=2, grid=32, n_spheres=4)
    acc = A.MakeAccelerator("ray-bvh", sc["tris"], {"walk": 1})
    o4, d4 = dev(S.random_rays(4096, -4.0, 4.0, seed=3))
    r = acc.autotune(o4, d4)
    assert len(r["candidates"]) == 1 and r["best"] == {"walk": 1}
    acc.close()


def test_autotune_rejects_bad_arguments(gpu_lib):
    import ctypes as C
    from pbrt_gb300 import _lib as L
    sc = S.terrain_icospheres(seed=2, grid=16, n_spheres=2)
    acc = A.MakeAccelerator("naive", sc["tris"])
    o4, d4 = dev(S.random_rays(64, -4.0, 4.0, seed=3))
    r = L.TuneResult()
    for query, n in ((4, 64), (0, 0)):  # an unknown query bit; an empty batch
        rc = L.lib().pbg_autotune(acc.handle, o4.data_ptr(), d4.data_ptr(), None, n, query, 1, C.byref(r), None)
        assert rc == L.PBG_ERR_INVALID_ARGUMENT
    acc.close()


@pytest.mark.parametrize("kind", ["naive", "rayhierarchy", "ray-bvh"])
def test_autotune_tiny_batches_and_empty_scenes(gpu_lib, oracle, kind):
    """One ray, and a scene without triangles: every shape still answers
    identically (and a miss for the empty scene)."""
    import torch
    sc = S.terrain_icospheres(seed=2, grid=16, n_spheres=2)
    for tris in (sc["tris"], np.zeros((0, 9), np.float32)):
        acc = A.MakeAccelerator(kind, tris)
        rays = S.random_rays(1, [-4, -1, -4], [4, 4, 4], seed=9)
        o4, d4 = dev(rays)
        for anyhit in (False, True):
            r = acc.autotune(o4, d4, anyhit=anyhit, reps=1)
            assert r["mismatches"] == 0 and len(r["candidates"]) == EXPECTED[kind]
        prim = torch.empty(1, dtype=torch.int32, device="cuda")
        t, b1, b2 = (torch.empty(1, device="cuda") for _ in range(3))
        acc.intersect_device(o4, d4, prim, t, b1, b2)
        torch.cuda.synchronize()
        want = oracle.nearest(tris, rays)[0] if len(tris) else np.array([-1], np.int32)
        np.testing.assert_array_equal(prim.cpu().numpy(), want)
        acc.close()
