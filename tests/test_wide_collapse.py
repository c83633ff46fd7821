"""The eight-wide collapse on the host cores (no GPU): a C++ check compiled
against the library's exported collapse_wide builds the two-wide tree of a
seeded scene, collapses it and verifies the record map, the node format and
that no ray reaches fewer records through the wide tree than through the
two-wide one (tests/native/wide_collapse_check.cpp)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from pbrt_gb300 import _lib as L
from pbrt_gb300 import scenes as S

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    L.lib()  # the library is built
    nvcc = shutil.which("nvcc")
    if nvcc is None:
        pytest.skip("CUDA toolkit not available")
    cuda_inc = Path(nvcc).resolve().parents[1] / "include"  # <toolkit>/bin/nvcc -> <toolkit>/include
    if not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("CUDA headers not available")
    exe = tmp_path_factory.mktemp("wide") / "wide_collapse_check"
    build = Path(L.LIB_PATH).parent
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(cuda_inc),
                    "-I", str(ROOT / "pbrt-v2_gb300" / "csrc"), str(ROOT / "tests" / "native" / "wide_collapse_check.cpp"),
                    "-o", str(exe), "-L", str(build), "-lpbrtgb300", f"-Wl,-rpath,{build}"], check=True)
    return exe


@pytest.mark.parametrize("scene", ["terrain", "spheres", "ties"])
def test_wide_collapse_reaches_every_record(checker, tmp_path, scene):
    if scene == "terrain":
        tris = S.terrain_icospheres(seed=2, grid=96, n_spheres=12)["tris"]
    elif scene == "spheres":
        tris = S.displaced_icospheres(seed=3, n_inst=40)["tris"]
    else:  # a grid of coplanar, touching triangles: flat boxes and shared edges
        g = np.stack(np.meshgrid(np.arange(40.0), np.arange(40.0)), -1).reshape(-1, 2)
        a = np.c_[g, np.zeros(len(g))]
        tris = np.concatenate([np.c_[a, a + [1, 0, 0], a + [0, 1, 0]],
                               np.c_[a + [1, 0, 0], a + [1, 1, 0], a + [0, 1, 0]]])
    f = tmp_path / "tris.f32"
    np.ascontiguousarray(tris, dtype=np.float32).tofile(f)
    out = subprocess.run([str(checker), str(f), "300"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    ok, nwide, nbin, vw, vb = out.stdout.split()
    assert ok == "ok" and int(nwide) < int(nbin) and float(vw) < float(vb)
