"""Scene construction on the device: the ray-bvh tree built by the GPU
builder (pbg_params.bvh_build = 0, the default) against the host builder
(bvh_build = 1) and the oracle, and scenes created from pbrt's mesh arrays
(pbg_scene_create_mesh) against scenes from packed triangles."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from pbrt_gb300 import _lib as L
from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def same_hits(a, b, label):
    np.testing.assert_array_equal(a[0], b[0], err_msg=label)
    h = a[0] >= 0
    for k in (1, 2, 3):
        np.testing.assert_array_equal(a[k][h].view(np.uint32), b[k][h].view(np.uint32), err_msg=label)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_device_tree_on_golden_cases(gpu_lib, case):
    g = load_golden(case)
    tris, rays = g["tris"], g["rays"]
    dev = A.MakeAccelerator("ray-bvh", tris, {"bvhBuild": 0})
    got = dev.Intersect(rays.copy())
    np.testing.assert_array_equal(got[0], g["prim"])
    h = g["prim"] >= 0
    np.testing.assert_array_equal(got[1][h], g["t"][h])
    np.testing.assert_array_equal(dev.IntersectP(rays) == ord("1"), g["occ"] == 1)


@pytest.mark.parametrize("seed,n", [(1, 1), (2, 3), (3, 4), (4, 5), (5, 9), (6, 200)])
def test_device_tree_small_scenes(gpu_lib, oracle, seed, n):
    g = np.random.default_rng(seed)
    tris = g.uniform(-2, 2, (n, 9)).astype(np.float32)
    rays = S.random_rays(4096, -3.0, 3.0, seed=seed)
    want = oracle.BVH(tris).nearest(rays)
    got = A.MakeAccelerator("ray-bvh", tris, {"bvhBuild": 0}).Intersect(rays.copy())
    same_hits(got, want, f"{n} triangles")


def test_device_tree_equals_host_tree_results(gpu_lib, oracle):
    """The 1,024,000-triangle path scene's generator at a smaller size and
    the terrain scene: device and host trees answer identically (and as the
    oracle) on incoherent rays; the device tree has the host tree's size
    within a few percent (the same SAH splits; only centroids in one bin
    split differently)."""
    for sc in (S.displaced_icospheres(seed=3, n_inst=80, box=16.0), S.terrain_icospheres(seed=2)):
        tris = sc["tris"]
        rays = S.random_rays(40000, -8.0, 8.0, seed=9)
        rays[7, ::2] = 3.0
        dev = A.MakeAccelerator("ray-bvh", tris, {"bvhBuild": 0})
        host = A.MakeAccelerator("ray-bvh", tris, {"bvhBuild": 1})
        a, b = dev.Intersect(rays.copy()), host.Intersect(rays.copy())
        same_hits(a, b, "device vs host tree")
        same_hits(a, oracle.BVH(tris).nearest(rays), "device tree vs oracle")
        np.testing.assert_array_equal(dev.IntersectP(rays), host.IntersectP(rays))
        nd, nh = dev.stats()["bvh_nodes"], host.stats()["bvh_nodes"]
        assert abs(nd - nh) <= 0.05 * nh, (nd, nh)


def grid_mesh(n=40, seed=3):
    """A height-field mesh with shared vertices, per-vertex uvs."""
    g = np.random.default_rng(seed)
    xs, zs = np.meshgrid(np.linspace(-4, 4, n), np.linspace(-4, 4, n))
    P = np.stack([xs.ravel(), g.uniform(-0.5, 0.5, n * n), zs.ravel()], 1).astype(np.float32)
    uv = np.stack([xs.ravel() / 8 + 0.5, zs.ravel() / 8 + 0.5], 1).astype(np.float32)
    idx = []
    for j in range(n - 1):
        for i in range(n - 1):
            a, b, c, d = j * n + i, j * n + i + 1, (j + 1) * n + i + 1, (j + 1) * n + i
            idx += [(a, b, c), (a, c, d)]
    return P, np.array(idx, np.int32), uv


@pytest.mark.parametrize("kind", ["naive", "ray-bvh", "rayhierarchy"])
def test_mesh_ingestion_equals_packed_triangles(gpu_lib, kind):
    P, vi, uv = grid_mesh()
    tris = P[vi].reshape(-1, 9)
    uvs = uv[vi].reshape(-1, 6)
    rays = S.random_rays(20000, [-4, -2, -4], [4, 2, 4], seed=12)
    mesh = A.MakeAcceleratorFromMesh(kind, P, vi, uv)
    packed = A.MakeAccelerator(kind, tris, uvs=uvs)
    a, b = mesh.Intersect(rays.copy()), packed.Intersect(rays.copy())
    same_hits(a, b, kind)
    assert (a[0] >= 0).sum() > 1000
    np.testing.assert_array_equal(mesh.IntersectP(rays), packed.IntersectP(rays))
    # the mesh's per-vertex uvs reach the hit geometry as the packed uvs do
    np.testing.assert_array_equal(mesh.HitGeometry(rays, *a), packed.HitGeometry(rays, *b))


def test_mesh_ingestion_rejects_bad_indices(gpu_lib):
    P, vi, _ = grid_mesh(8)
    vi = vi.copy()
    vi[5, 1] = len(P)  # one past the last vertex
    for kind in ("naive", "ray-bvh", "rayhierarchy"):
        with pytest.raises(L.PbgError) as e:
            A.MakeAcceleratorFromMesh(kind, P, vi)
        assert e.value.status == L.PBG_ERR_INVALID_ARGUMENT
