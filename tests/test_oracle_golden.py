"""The CPU restatement (oracle/pbrt_oracle.c) against the reference's own
answers (tests/golden/*.npz, made by tests/golden/make_golden.py from the
pbrt-v2 sources): bit for bit."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_nearest_bit_exact(oracle, case):
    g = load_golden(case)
    prim, t, b1, b2 = oracle.nearest(g["tris"], g["rays"], threads=4)
    np.testing.assert_array_equal(prim, g["prim"])
    hit = prim >= 0
    # bit patterns, not just values
    np.testing.assert_array_equal(t[hit].view(np.uint32), g["t"][hit].view(np.uint32))
    np.testing.assert_array_equal(b1[hit], g["b1"][hit])
    np.testing.assert_array_equal(b2[hit], g["b2"][hit])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_anyhit_bit_exact(oracle, case):
    g = load_golden(case)
    occ = oracle.anyhit(g["tris"], g["rays"], threads=4)
    np.testing.assert_array_equal(occ, g["occ"])


def test_shadow_rays(oracle):
    g = load_golden("sphere_small")
    occ = oracle.anyhit(g["tris"], g["shadow_rays"], threads=4)
    np.testing.assert_array_equal(occ, g["shadow_occ"])


@pytest.mark.parametrize("case", ["sphere_small", "soup"])
def test_hit_geometry(oracle, case):
    g = load_golden(case)
    uvs = g.get("uvs")
    geo = oracle.hits_geometry(g["tris"], uvs, g["rays"], g["prim"], g["t"], g["b1"], g["b2"])
    np.testing.assert_array_equal(geo, g["geo"])


@pytest.mark.parametrize("case", ["sphere_small", "soup", "degenerate"])
def test_bvh_baseline_equals_brute_force(oracle, case):
    """The timed CPU baseline (SAH BVH port) answers like the in-order loop."""
    g = load_golden(case)
    B = oracle.BVH(g["tris"])
    prim, t, b1, b2 = B.nearest(g["rays"], threads=4)
    np.testing.assert_array_equal(prim, g["prim"])
    np.testing.assert_array_equal(t[prim >= 0], g["t"][prim >= 0])
    np.testing.assert_array_equal(B.anyhit(g["rays"], threads=4), g["occ"])


def test_valid_mask(oracle):
    g = load_golden("soup")
    valid = (np.arange(g["rays"].shape[1]) % 3 != 0).astype(np.uint8)
    prim, t, _, _ = oracle.nearest(g["tris"], g["rays"], valid=valid, threads=2)
    assert (prim[valid == 0] == -1).all()
    np.testing.assert_array_equal(prim[valid == 1], g["prim"][valid == 1])
    occ = oracle.anyhit(g["tris"], g["rays"], valid=valid, threads=2)
    assert (occ[valid == 0] == 0).all()


def test_planted_mistake_is_caught(oracle):
    """A wrong answer planted in the oracle's output is seen by the check."""
    g = load_golden("sphere_small")
    prim, t, _, _ = oracle.nearest(g["tris"], g["rays"], threads=4)
    i = int(np.flatnonzero(prim >= 0)[0])
    prim[i] = (prim[i] + 1) % len(g["tris"])
    assert not np.array_equal(prim, g["prim"])
