"""Many scenes in one launch (pbg_sceneset_*): every scene's answers must be
bit-identical to the single-scene ray-bvh kernels and to the golden answers,
whatever the tile, the launch shape, the graph replay or the scene order."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

torch = pytest.importorskip("torch")


def to_o4d4(rays):
    o4 = np.ascontiguousarray(np.stack([rays[0], rays[1], rays[2], rays[6]], 1).astype(np.float32))
    d4 = np.ascontiguousarray(np.stack([rays[3], rays[4], rays[5], rays[7]], 1).astype(np.float32))
    return o4, d4


def offsets(counts):
    return np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)


class Packed:
    """Scene-after-scene device arrays for a list of (near, shadow) batches."""

    def __init__(self, near_list, shadow_list):
        self.near_off = offsets([r.shape[1] for r in near_list])
        self.occ_off = offsets([r.shape[1] for r in shadow_list])
        cat = lambda lst: np.concatenate(lst, 1) if lst else np.zeros((8, 0), np.float32)
        on, dn = to_o4d4(cat(near_list))
        os_, ds = to_o4d4(cat(shadow_list))
        dev = "cuda"
        self.o4n, self.d4n = torch.from_numpy(on).to(dev), torch.from_numpy(dn).to(dev)
        self.o4s, self.d4s = torch.from_numpy(os_).to(dev), torch.from_numpy(ds).to(dev)
        nn, ns = int(self.near_off[-1]), int(self.occ_off[-1])
        self.prim = torch.full((nn,), -7, dtype=torch.int32, device=dev)
        self.t = torch.full((nn,), -7.0, device=dev)
        self.b1 = torch.full((nn,), -7.0, device=dev)
        self.b2 = torch.full((nn,), -7.0, device=dev)
        self.occ = torch.full((ns,), 7, dtype=torch.uint8, device=dev)

    def args(self):
        return dict(o4n=self.o4n, d4n=self.d4n, near_offsets=self.near_off, prim=self.prim, t=self.t,
                    b1=self.b1, b2=self.b2, o4s=self.o4s, d4s=self.d4s, occ_offsets=self.occ_off,
                    occ=self.occ)

    def results(self):
        torch.cuda.synchronize()
        return (self.prim.cpu().numpy(), self.t.cpu().numpy(), self.b1.cpu().numpy(),
                self.b2.cpu().numpy(), self.occ.cpu().numpy())


def per_scene(tris, near, shadow):
    """The plain single-scene ray-bvh kernels on one scene."""
    acc = A.MakeAccelerator("ray-bvh", tris)
    n, m = near.shape[1], shadow.shape[1]
    on, dn = to_o4d4(near)
    os_, ds = to_o4d4(shadow)
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    t, b1, b2 = (torch.empty(n, device="cuda") for _ in range(3))
    occ = torch.empty(m, dtype=torch.uint8, device="cuda")
    if n:
        acc.intersect_device(torch.from_numpy(on).cuda(), torch.from_numpy(dn).cuda(), prim, t, b1, b2)
    if m:
        acc.occluded_device(torch.from_numpy(os_).cuda(), torch.from_numpy(ds).cuda(), occ)
    torch.cuda.synchronize()
    return prim.cpu().numpy(), t.cpu().numpy(), b1.cpu().numpy(), b2.cpu().numpy(), occ.cpu().numpy()


def assert_scene_equal(got, want, label, bitwise=True):
    """prim and t bit for bit; b1/b2 bit for bit against the same kernels, by
    value against the golden answers (which may hold +0 where the exact
    test rounds to -0, as the single-scene parity tests allow)."""
    prim, t, b1, b2 = got
    wprim, wt, wb1, wb2 = want
    bad = np.flatnonzero(prim != wprim)
    assert bad.size == 0, f"{label}: {bad.size} prim mismatches, first {bad[:8]}"
    h = prim >= 0
    np.testing.assert_array_equal(t[h].view(np.uint32), wt[h].view(np.uint32), err_msg=label)
    if bitwise:
        np.testing.assert_array_equal(b1[h].view(np.uint32), wb1[h].view(np.uint32), err_msg=label)
        np.testing.assert_array_equal(b2[h].view(np.uint32), wb2[h].view(np.uint32), err_msg=label)
    else:
        np.testing.assert_array_equal(b1[h], wb1[h], err_msg=label)
        np.testing.assert_array_equal(b2[h], wb2[h], err_msg=label)
    assert np.all(t[~h] == 0) and np.all(b1[~h] == 0) and np.all(b2[~h] == 0), label


@pytest.mark.gpu
def test_golden_scenes_in_one_set(gpu_lib):
    """All golden cases as one set: nearest and any-hit answers equal the
    reference's golden ones, scene by scene."""
    from pbrt_gb300.batch import SceneSet
    gs = [load_golden(c) for c in GOLDEN_CASES]
    sset = SceneSet([g["tris"] for g in gs])
    pk = Packed([g["rays"] for g in gs], [g["rays"] for g in gs])
    for tile, walk in ((32, 1), (64, 1), (256, 1), (64, 2), (64, 3), (64, 4)):
        for graph in (False, True):
            sset.trace(**pk.args(), tile=tile, use_graph=graph, walk=walk)
            prim, t, b1, b2, occ = pk.results()
            for k, (c, g) in enumerate(zip(GOLDEN_CASES, gs)):
                a, b = pk.near_off[k], pk.near_off[k + 1]
                assert_scene_equal((prim[a:b], t[a:b], b1[a:b], b2[a:b]),
                                   (g["prim"], g["t"], g["b1"], g["b2"]), f"{c} tile {tile}",
                                   bitwise=False)
                a, b = pk.occ_off[k], pk.occ_off[k + 1]
                np.testing.assert_array_equal(occ[a:b], (g["occ"] == 1).astype(np.uint8), err_msg=c)
    sset.close()


def small_set(seed=9, n=5):
    return S.many_scenes(seed=seed, n_scenes=n, median_tris=3000, sigma=0.8,
                         tri_range=(500, 20000), ray_range=(1000, 9000))


@pytest.mark.gpu
def test_matches_per_scene_kernels(gpu_lib):
    """Generated scenes (primary, path and shadow rays) against the plain
    per-scene ray-bvh kernels, bit for bit; graph replay on the second call;
    per-scene completion times reported for every scene."""
    from pbrt_gb300.batch import SceneSet
    scs = small_set()
    sset = SceneSet([s["tris"] for s in scs])
    pk = Packed([s["near"] for s in scs], [s["shadow"] for s in scs])
    st1, per1 = sset.trace(**pk.args(), stats=True)
    got = pk.results()
    st2, per2 = sset.trace(**pk.args(), stats=True)
    assert st2["graph_replayed"] and not st1["graph_replayed"]
    got2 = pk.results()
    for a, b in zip(got, got2):
        np.testing.assert_array_equal(a, b)
    for k, s in enumerate(scs):
        want = per_scene(s["tris"], s["near"], s["shadow"])
        a, b = pk.near_off[k], pk.near_off[k + 1]
        assert_scene_equal(tuple(x[a:b] for x in got[:4]), want[:4], f"scene {k}")
        a, b = pk.occ_off[k], pk.occ_off[k + 1]
        np.testing.assert_array_equal(got[4][a:b], want[4], err_msg=f"scene {k} occ")
    hits = (got[0] >= 0).mean()
    assert 0.2 < hits <= 1.0  # the camera and path rays do meet the terrain
    assert st1["rays"] == int(pk.near_off[-1] + pk.occ_off[-1])
    assert np.all(per1 > 0) and st1["scene_ms_p50"] <= st1["scene_ms_p99"] <= st1["ms"] * 1.5 + 1.0
    sset.close()


@pytest.mark.gpu
def test_trace_host_in_two_halves(gpu_lib):
    """trace_host: pinned host rays in and results out, in two halves of the
    scenes whose copies overlap the other half's trace; both halves' graphs
    stay cached; bit for bit the answers of one device-buffer trace, for
    several split points."""
    from pbrt_gb300.batch import SceneSet
    scs = small_set()
    sset = SceneSet([s["tris"] for s in scs])
    pk = Packed([s["near"] for s in scs], [s["shadow"] for s in scs])
    sset.trace(**pk.args())
    want = pk.results()
    pin = lambda x: x.cpu().pin_memory()
    host = dict(o4n=pin(pk.o4n), d4n=pin(pk.d4n), o4s=pin(pk.o4s), d4s=pin(pk.d4s),
                prim=pin(pk.prim), t=pin(pk.t), b1=pin(pk.b1), b2=pin(pk.b2), occ=pin(pk.occ))
    stream, copy_stream = torch.cuda.Stream(), torch.cuda.Stream(priority=-1)
    for split in (None, 1, len(scs) - 1):
        for key in ("prim", "t", "b1", "b2", "occ"):
            host[key].fill_(0)
        dev = dict(o4n=torch.zeros_like(pk.o4n), d4n=torch.zeros_like(pk.d4n), o4s=torch.zeros_like(pk.o4s),
                   d4s=torch.zeros_like(pk.d4s), prim=torch.full_like(pk.prim, -7), t=torch.full_like(pk.t, -7.0),
                   b1=torch.full_like(pk.b1, -7.0), b2=torch.full_like(pk.b2, -7.0), occ=torch.full_like(pk.occ, 7))
        for _ in range(2):  # the second call replays both halves' graphs
            sset.trace_host(host, dev, pk.near_off, pk.occ_off, stream, copy_stream, split=split)
            got = tuple(host[k].numpy() for k in ("prim", "t", "b1", "b2", "occ"))
            for a, b in zip(got, want):
                np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8), err_msg=f"split {split}")
    sset.close()


@pytest.mark.gpu
def test_empty_and_ragged(gpu_lib):
    """Scenes with no triangles, scenes with no rays of one kind, one-ray
    scenes, and a call with no any-hit rays at all."""
    from pbrt_gb300.batch import SceneSet
    scs = small_set(seed=11, n=3)
    empty = np.zeros((0, 9), np.float32)
    tris = [scs[0]["tris"], empty, scs[1]["tris"], scs[2]["tris"]]
    near = [scs[0]["near"][:, :1], scs[1]["near"][:, :77], np.zeros((8, 0), np.float32),
            scs[2]["near"]]
    shad = [np.zeros((8, 0), np.float32), scs[1]["shadow"][:, :33], scs[1]["shadow"],
            scs[2]["shadow"][:, :1]]
    sset = SceneSet(tris)
    pk = Packed(near, shad)
    sset.trace(**pk.args(), tile=96, threads=64, ctas_per_sm=2, use_graph=False)
    got = pk.results()
    pk.prim.fill_(-7)
    pk.occ.fill_(7)
    sset.trace(**pk.args(), threads=64, ctas_per_sm=1, use_graph=False, walk=2)
    got_p = pk.results()
    for a, b in zip(got, got_p):
        np.testing.assert_array_equal(a, b)
    for walk in (3, 4):  # the eight-wide trees, one launch per query kind
        pk.prim.fill_(-7)
        pk.occ.fill_(7)
        sset.trace(**pk.args(), ctas_per_sm=1, use_graph=False, walk=walk)
        for a, b in zip(got, pk.results()):
            np.testing.assert_array_equal(a, b)
    for k in range(4):
        want = per_scene(tris[k], near[k], shad[k])
        a, b = pk.near_off[k], pk.near_off[k + 1]
        assert_scene_equal(tuple(x[a:b] for x in got[:4]), want[:4], f"scene {k}")
        a, b = pk.occ_off[k], pk.occ_off[k + 1]
        np.testing.assert_array_equal(got[4][a:b], want[4])
    assert np.all(got[0][pk.near_off[1]:pk.near_off[2]] == -1)  # empty scene: misses
    # nearest-hit only
    pk2 = Packed(near, [np.zeros((8, 0), np.float32)] * 4)
    sset.trace(o4n=pk2.o4n, d4n=pk2.d4n, near_offsets=pk2.near_off, prim=pk2.prim, t=pk2.t,
               b1=pk2.b1, b2=pk2.b2)
    got2 = pk2.results()
    np.testing.assert_array_equal(got2[0], got[0])
    sset.close()


@pytest.mark.gpu
def test_autotune_and_bad_arguments(gpu_lib):
    from pbrt_gb300 import _lib as L
    from pbrt_gb300.batch import SceneSet
    scs = small_set(seed=13, n=3)
    sset = SceneSet([s["tris"] for s in scs])
    pk = Packed([s["near"] for s in scs], [s["shadow"] for s in scs])
    best = sset.autotune(**pk.args())
    assert best["tile"] in (32, 64, 128, 256) and best["threads"] in (64, 128, 256)
    assert best["ctas_per_sm"] >= 1 and best["walk"] in (1, 2, 3, 4)
    st, _ = sset.trace(**pk.args(), stats=True)
    assert (st["tile"], st["threads"], st["ctas_per_sm"], st["walk"]) == (
        best["tile"], best["threads"], best["ctas_per_sm"], best["walk"])
    got = pk.results()
    for k, s in enumerate(scs):
        want = per_scene(s["tris"], s["near"], s["shadow"])
        a, b = pk.near_off[k], pk.near_off[k + 1]
        np.testing.assert_array_equal(got[0][a:b], want[0])
    with pytest.raises(L.PbgError) as e:
        sset.trace(**pk.args(), tile=48)
    assert e.value.status == L.PBG_ERR_INVALID_ARGUMENT
    bad = pk.args()
    bad["near_offsets"] = pk.near_off[::-1].copy()
    with pytest.raises(L.PbgError):
        sset.trace(**bad)
    bad = pk.args()
    bad["prim"] = None
    with pytest.raises(L.PbgError):
        sset.trace(**bad)
    sset.close()


def test_many_scenes_generator_is_seeded():
    a = S.many_scenes(seed=21, n_scenes=3, median_tris=2000, tri_range=(500, 4000),
                      ray_range=(500, 1500))
    b = S.many_scenes(seed=21, n_scenes=3, median_tris=2000, tri_range=(500, 4000),
                      ray_range=(500, 1500))
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x["tris"], y["tris"])
        np.testing.assert_array_equal(x["near"], y["near"])
        np.testing.assert_array_equal(x["shadow"], y["shadow"])
        n_prim, n_path, n_shad = x["kinds"]
        assert x["near"].shape[1] == n_prim + n_path and x["shadow"].shape[1] == n_shad
        s = x["shadow"]
        assert np.all(s[7] > s[6]) and np.all(np.isfinite(s[:6]))
