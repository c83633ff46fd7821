"""Cluster-ordered any-hit walks (ray-bvh): what an ordering gains, counted.

Shadow rays leave surface points of the displaced-icosphere scene towards
an area light above it.  The plain walk (nearest child first) must find any
occluder; an ordered walk visits one predicted cluster (a subtree of the
BVH's top cut) first and stops there when it holds an occluder.  Counted
with the traversal kernels' counting variant (profiling level 2):
  * perfect hints -- each ray's own occluder cluster, from the plain walk --
    bound what any ordering can save;
  * the learned ordering, trained online on occluder clusters of earlier
    shadow batches, must visit fewer nodes than the plain walk.
Occlusion is identical in every mode."""
import numpy as np
import pytest

from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

pytestmark = pytest.mark.gpu

LIGHT = np.array([[-6, 14, -6], [6, 14, -6], [6, 14, 6], [-6, 14, 6]], np.float32)


def shadow_batch(acc, seed, n=65536):
    """Shadow segments from the hit points of random rays to random points
    on the light (mint = 1e-3 t, maxt = 0.999 of the distance)."""
    import torch
    rays = S.random_rays(n, -8.0, 8.0, seed=seed)
    prim, t, _, _ = acc.Intersect(rays.copy())
    hit = prim >= 0
    g = np.random.default_rng(seed + 1)
    p = rays[0:3] + rays[3:6] * np.where(hit, t, 0)[None]
    u, v = g.random(n), g.random(n)
    lp = (LIGHT[0][:, None] + (LIGHT[1] - LIGHT[0])[:, None] * u[None] + (LIGHT[3] - LIGHT[0])[:, None] * v[None])
    d = lp - p
    dist = np.sqrt((d ** 2).sum(0))
    dist = np.where(dist > 0, dist, 1.0)
    o4 = np.stack([p[0], p[1], p[2], np.where(hit, 1e-3 * t, 0.0)], 1).astype(np.float32)
    d4 = np.stack([d[0] / dist, d[1] / dist, d[2] / dist, dist * 0.999], 1).astype(np.float32)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return dev(o4), dev(d4), dev(hit.astype(np.uint8))


def counted(acc, fn):
    import torch
    acc.profile(2)
    fn()
    torch.cuda.synchronize()
    w = acc.stats()["work"]
    acc.profile(False)
    return w


def scene():
    sc = S.displaced_icospheres(seed=3, n_inst=60, box=16.0)
    return A.MakeAccelerator("ray-bvh", sc["tris"])


def test_perfect_hints_bound_the_anyhit_gain(gpu_lib):
    import torch
    acc = scene()
    o4, d4, valid = shadow_batch(acc, 7)
    n = o4.shape[0]
    occ0 = torch.empty(n, dtype=torch.uint8, device="cuda")
    occluder = torch.empty(n, dtype=torch.int32, device="cuda")
    w0 = counted(acc, lambda: acc.occluded_hinted_device(o4, d4, None, occ0, occluder, valid=valid))
    hint = torch.empty(n, dtype=torch.int16, device="cuda")
    acc.clusters_of_device(occluder, hint)
    occ1 = torch.empty_like(occ0)
    w1 = counted(acc, lambda: acc.occluded_hinted_device(o4, d4, hint, occ1, valid=valid))
    assert torch.equal(occ0, occ1)
    blocked = int(occ0.sum())
    assert 0.2 * n < blocked < 0.9 * n  # a batch with both answers
    # every occluder lies in a cluster; valid occluded rays get a hint
    h = hint.view(torch.int16).cpu().numpy().view(np.uint16)
    assert np.all((h < 256) == (occ0.cpu().numpy() == 1))
    # the ceiling: a perfect first guess saves node tests and triangle tests
    assert w1["node_tests"] < 0.8 * w0["node_tests"], (w0, w1)
    assert w1["filter_tests"] < w0["filter_tests"], (w0, w1)
    # results also unchanged with hints that point at the wrong clusters
    wrong = torch.randint(0, 256, (n,), dtype=torch.int32, device="cuda").to(torch.int16)
    occ2 = torch.empty_like(occ0)
    acc.occluded_hinted_device(o4, d4, wrong, occ2, valid=valid)
    torch.cuda.synchronize()
    assert torch.equal(occ0, occ2)
    acc.close()


def test_trained_ordering_cuts_anyhit_work(gpu_lib):
    import torch
    acc = scene()
    acc.learn_enable(True, batch=4096, steps_per_train=40, lr=0.1, seed=5, queries=2)
    for k in range(6):  # shadow batches: occluder records, then SGD steps
        o4, d4, valid = shadow_batch(acc, 100 + k)
        occ = torch.empty(o4.shape[0], dtype=torch.uint8, device="cuda")
        acc.occluded_device(o4, d4, occ, valid=valid)
        acc.learn_train(0)
    st = acc.learn_stats()
    assert st["trained_steps"] >= 200 and st["records"] > 0
    o4, d4, valid = shadow_batch(acc, 7)
    n = o4.shape[0]
    occ_l = torch.empty(n, dtype=torch.uint8, device="cuda")
    w_learned = counted(acc, lambda: acc.occluded_device(o4, d4, occ_l, valid=valid))
    acc.learn_enable(False)
    occ_p = torch.empty_like(occ_l)
    w_plain = counted(acc, lambda: acc.occluded_device(o4, d4, occ_p, valid=valid))
    assert torch.equal(occ_l, occ_p)
    assert w_learned["node_tests"] < w_plain["node_tests"], (w_plain, w_learned)
    acc.close()
