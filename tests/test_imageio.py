"""Film output (PFM) and the exrdiff-style comparator (pbrt_gb300.imageio)."""
import os
import tempfile

import numpy as np
import pytest

from conftest import load_golden
from pbrt_gb300 import imageio as I


def test_pfm_round_trip_and_header(tmp_path):
    img = np.random.default_rng(3).random((5, 7, 3)).astype(np.float32)
    p = tmp_path / "a.pfm"
    I.write_pfm(str(p), img)
    raw = p.read_bytes()
    assert raw.startswith(b"PF\n7 5\n-1.000000\n")
    assert len(raw) == len(b"PF\n7 5\n-1.000000\n") + 5 * 7 * 3 * 4
    np.testing.assert_array_equal(I.read_pfm(str(p)), img)


def test_pfm_bytes_equal_the_reference_writer(oracle):
    """The reference's own PFM of a breadth-first render, written again by
    write_pfm, is byte for byte the same file."""
    if not oracle.ref_available():
        pytest.skip("reference build not present")
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import bf_scene_text
    from pbrt_gb300 import scenes as S
    base = S.config_small_naive()["tris"]
    point = 'LightSource "point" "point from" [0 3 0] "rgb I" [8 8 8]\n'
    with tempfile.TemporaryDirectory() as td:
        img = oracle.ref_render(bf_scene_text(base, "directlighting", point), td)
        theirs = open(os.path.join(td, "out.pfm"), "rb").read()
        I.write_pfm(os.path.join(td, "mine.pfm"), img)
        mine = open(os.path.join(td, "mine.pfm"), "rb").read()
    assert mine == theirs


def test_image_diff_thresholds():
    a = load_golden("render_bf")["image_direct"]
    r = I.image_diff(a, a.copy())
    assert not r["differ"] and r["small"] == 0 and r["big"] == 0 and r["mse"] == 0.0
    b = a.copy()
    b[3, 4, 1] *= 1.01  # one value 1% off: small, not big
    b[10, 20, 0] *= 1.2  # one value 20% off: small and big
    r = I.image_diff(a, b)
    nz = int(np.count_nonzero(a[3, 4, 1])) + int(np.count_nonzero(a[10, 20, 0]))
    assert r["differ"] and r["small"] == nz and r["big"] == int(np.count_nonzero(a[10, 20, 0]))
    # with a tolerance on the average delta the same images pass
    assert not I.image_diff(a, b, tol=1.0)["differ"]
    assert I.image_diff(a, a[:-1])["differ"]


def test_cli_exit_codes(tmp_path):
    a = load_golden("render_bf")["image_path"]
    pa, pb, pd = tmp_path / "a.pfm", tmp_path / "b.pfm", tmp_path / "d.pfm"
    I.write_pfm(str(pa), a)
    I.write_pfm(str(pb), a)
    assert I.main([str(pa), str(pb)]) == 0
    I.write_pfm(str(pb), a * 1.5)
    assert I.main([str(pa), str(pb), "-o", str(pd)]) == 1
    np.testing.assert_array_equal(I.read_pfm(str(pd)), np.abs(a - (a * 1.5).astype(np.float32)))
