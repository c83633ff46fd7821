"""The breadth-first renderer: the oracle's restatement against the
reference's own render, and the GPU wavefront against both.  Image bar:
RMSE <= 1e-4 (the GPU and the oracle are expected to agree exactly)."""
import numpy as np
import pytest

from conftest import load_golden
from pbrt_gb300 import accel as A
from pbrt_gb300 import render as R
from pbrt_gb300 import scenes as S

RMSE_TOL = 1e-4


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


def test_oracle_render_equals_reference_render(oracle):
    """Small naive workload (256x256, 1 spp at pixel centres, point light,
    matte 0.7, directlighting): the oracle restatement reproduces the image
    pbrt itself rendered (tests/golden/render_small.npz)."""
    g = load_golden("render_small")
    cfg = S.config_small_naive()
    img = oracle.render(cfg["tris"], g["r2c"], g["c2w"], 256, 256,
                        [{"type": "point", "pos": g["light_pos"], "I": g["light_I"]}])
    assert rmse(img, g["image"]) <= RMSE_TOL
    np.testing.assert_array_equal(img, g["image"])


def test_camera_matrices_restated():
    """perspective_camera (used for the synthetic workloads) against the
    reference camera's matrices: CameraToWorld exact, RasterToCamera within
    one ulp of its largest entry."""
    g = load_golden("render_small")
    r2c, c2w = R.perspective_camera(256, 256, (0.0, 1.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 45.0)
    np.testing.assert_array_equal(c2w, g["c2w"])
    assert np.abs(r2c - g["r2c"]).max() <= 1e-6 * np.abs(g["r2c"]).max()


def small_area_scene():
    sc = S.terrain_icospheres(seed=2, grid=48, n_spheres=6)
    r2c, c2w = R.perspective_camera(64, 48, (0.0, 9.0, -14.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 50.0)
    quad = sc["area_light_quad"]
    return sc["tris"], r2c, c2w, quad


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["naive", "ray-bvh", "rayhierarchy"])
def test_gpu_render_equals_reference_render(gpu_lib, kind):
    g = load_golden("render_small")
    cfg = S.config_small_naive()
    acc = A.MakeAccelerator(kind, cfg["tris"])
    acc.Preprocess(None, 1, 1, 1, xres=256, yres=256)
    cam = R.camera_struct(g["r2c"], g["c2w"], 256, 256)
    img, st = R.render(acc, cam, [R.point_light(g["light_pos"], g["light_I"])],
                       R.render_params("directlighting"))
    assert st["camera_rays"] == 65536
    assert rmse(img, g["image"]) <= RMSE_TOL
    np.testing.assert_array_equal(img, g["image"])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["ray-bvh", "rayhierarchy"])
def test_gpu_direct_area_light_equals_oracle(gpu_lib, oracle, kind):
    """Area light with 4 samples per hit, 2x2 jittered spp (the ray-hierarchy
    workload at small size)."""
    tris, r2c, c2w, quad = small_area_scene()
    acc = A.MakeAccelerator(kind, tris)
    cam = R.camera_struct(r2c, c2w, 64, 48)
    lt = R.quad_light(quad, (40.0, 40.0, 40.0), nsamples=4)
    prm = R.render_params("directlighting", spp=(2, 2), jitter=True, seed=5)
    img, st = R.render(acc, cam, [lt], prm)
    want = oracle.render(tris, r2c, c2w, 64, 48,
                         [{"type": "quad", "quad": quad, "L": (40.0, 40.0, 40.0), "nsamples": 4}],
                         spp=(2, 2), jitter=True, seed=5)
    assert img.mean() > 0.01
    assert rmse(img, want) <= RMSE_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["ray-bvh", "rayhierarchy"])
def test_gpu_path_equals_oracle(gpu_lib, oracle, kind):
    """Path tracing to depth 5 with Russian roulette after bounce 3 on
    displaced icospheres (the ray-bvh workload at small size)."""
    sc = S.displaced_icospheres(seed=3, n_inst=40, box=12.0)
    tris = sc["tris"]
    r2c, c2w = R.perspective_camera(48, 48, (0.0, 0.0, -16.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0)
    quad = np.array([[-3, 9, -3], [3, 9, -3], [3, 9, 3], [-3, 9, 3]], np.float32)
    acc = A.MakeAccelerator(kind, tris)
    cam = R.camera_struct(r2c, c2w, 48, 48)
    prm = R.render_params("path", spp=(2, 2), jitter=True, seed=9, max_depth=5)
    img, st = R.render(acc, cam, [R.quad_light(quad, (30.0, 30.0, 30.0), 1)], prm)
    want = oracle.render(tris, r2c, c2w, 48, 48,
                         [{"type": "quad", "quad": quad, "L": (30.0, 30.0, 30.0), "nsamples": 1}],
                         integrator="path", spp=(2, 2), jitter=True, seed=9, max_depth=5)
    assert st["bounces"] >= 2
    assert img.mean() > 0.001
    assert rmse(img, want) <= RMSE_TOL


@pytest.mark.gpu
def test_overlapped_bounces_equal_serial(gpu_lib, oracle):
    """Path frames on ray-bvh and naive scenes trace each bounce's shadow
    rays on a second stream beside the next bounce's nearest-hit rays;
    rayhierarchy frames stay serial.  All three images are identical (the
    resolves still add to each path's radiance in bounce order) and equal
    the oracle's."""
    sc = S.displaced_icospheres(seed=3, n_inst=24, box=12.0)
    tris = sc["tris"]
    r2c, c2w = R.perspective_camera(96, 80, (0.0, 0.0, -16.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0)
    quad = np.array([[-3, 9, -3], [3, 9, -3], [3, 9, 3], [-3, 9, 3]], np.float32)
    cam = R.camera_struct(r2c, c2w, 96, 80)
    prm = R.render_params("path", spp=(2, 2), jitter=True, seed=21, max_depth=5)
    light = R.quad_light(quad, (30.0, 30.0, 30.0), 1)
    imgs = {}
    for kind in ("ray-bvh", "naive", "rayhierarchy"):
        acc = A.MakeAccelerator(kind, tris)
        for _ in range(2):  # a second frame reuses the kept buffers and streams
            imgs[kind], st = R.render(acc, cam, [light], prm)
        assert st["bounces"] >= 3
        acc.close()
    np.testing.assert_array_equal(imgs["ray-bvh"], imgs["rayhierarchy"])
    np.testing.assert_array_equal(imgs["naive"], imgs["rayhierarchy"])
    want = oracle.render(tris, r2c, c2w, 96, 80,
                         [{"type": "quad", "quad": quad, "L": (30.0, 30.0, 30.0), "nsamples": 1}],
                         integrator="path", spp=(2, 2), jitter=True, seed=21, max_depth=5)
    assert rmse(imgs["ray-bvh"], want) <= RMSE_TOL
