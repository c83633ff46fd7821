"""Image parity with the reference's own breadth-first renders.

tests/golden/render_bf.npz holds images that pbrt itself rendered
(oracle/_ref/pbrt_ref, Renderer "breadth-first", Accelerator "naive" through
the CPU batch backend of oracle/ref): a 48x40 image, 2x2 jittered stratified
samples, the small sphere workload lit by a 2-triangle AreaLightSource
"diffuse" that the camera sees (directlighting with 4 light samples; path
to depth 5) or by a point light.  The renderer and the oracle are fed the
reference's own sample stream -- one task's StratifiedSampler output and
the continuation of its RNG(0), restated in oracle/pbrt_sampler.c and pinned
here against pbrt's own values -- so they must reproduce pbrt's image:
bar RMSE <= 1e-4.  Directlighting and the point light are exact; path
tracing differs only where the host libm's cosf / sinf are not correctly
rounded (about 0.1% of angles, one ulp of a direction)."""
import numpy as np
import pytest

from conftest import load_golden
from pbrt_gb300 import accel as A
from pbrt_gb300 import render as R
from pbrt_gb300 import scenes as S

RMSE_TOL = 1e-4
XRES, YRES, SPP, MAX_DEPTH, NSAMPLES, L_AREA = 48, 40, (2, 2), 5, 4, (5.0, 5.0, 5.0)
EXTENT = (0, XRES + 1, 0, YRES + 1)  # ImageFilm's sample extent with the 0.5 box filter


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


def scene(kind):
    base = S.config_small_naive()["tris"]
    if kind == "point":
        return base, [{"type": "point", "pos": (0.0, 3.0, 0.0), "I": (8.0, 8.0, 8.0)}]
    q = load_golden("render_bf")["quad"]
    light = np.array([np.r_[q[0], q[1], q[2]], np.r_[q[0], q[2], q[3]]], np.float32)
    ns = NSAMPLES if kind == "direct" else 1
    return (np.concatenate([base, light]).astype(np.float32),
            [{"type": "mesh", "first": len(base), "ntri": 2, "L": L_AREA, "nsamples": ns}])


def integrator(kind):
    return "path" if kind == "path" else "directlighting"


def stream(oracle, kind):
    """The task's samples as the renderer takes them (pbg_sample_stream)."""
    integ = integrator(kind)
    nsl = [1] if kind != "direct" else [NSAMPLES]
    n1d, n2d = R.sample_arrays(integ, nsl)
    count = XRES * YRES * SPP[0] * SPP[1]
    nrng = 11 * count * (MAX_DEPTH - 2) if integ == "path" else 1
    img, o1, o2, rng = oracle.pbrt_task_samples(EXTENT, SPP, n1d, n2d, count, nrng)
    return img, R.stream_dims(integ, nsl, o1, o2), rng


@pytest.mark.parametrize("tag,integ,ns", [("path", "path", 1), ("direct", "directlighting", NSAMPLES)])
def test_sampler_restatement_equals_reference_samples(oracle, tag, integ, ns):
    """oracle/pbrt_sampler.c reproduces pbrt's StratifiedSampler + RNG bit for
    bit: against the fixture's first 64 samples and 2048 RNG draws, and, where
    the reference build exists, against a whole task of pbrt's own."""
    g = load_golden("render_bf")
    n1d, n2d = R.sample_arrays(integ, [ns])
    got = oracle.pbrt_task_samples(EXTENT, SPP, n1d, n2d, 64, 2048)
    for a, key in zip(got, ("img", "oned", "twod", "rng")):
        np.testing.assert_array_equal(a, g[f"samp_{tag}_{key}"])
    if oracle.ref_available():
        count = XRES * YRES * SPP[0] * SPP[1]
        mine = oracle.pbrt_task_samples(EXTENT, SPP, n1d, n2d, count, 50000)
        theirs = oracle.pbrt_task_samples(EXTENT, SPP, n1d, n2d, count, 50000, reference=True)
        for a, b in zip(mine, theirs):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("tag", ["quad", "uneven"])
def test_area_light_restatement_equals_reference(oracle, tag):
    """The restated DiffuseAreaLight::Sample_L over a triangle ShapeSet (its
    area CDF, the reversed shape order of the ShapeSet's refinement, the
    re-intersection and the summed pdf) gives pbrt's radiance, direction, pdf
    and shadow segment bit for bit."""
    g = load_golden("render_bf")
    got = oracle.area_light_sample(g[f"light_{tag}_tris"], L_AREA, g[f"light_{tag}_q"])
    np.testing.assert_array_equal(got.view(np.uint32), g[f"light_{tag}_out"].view(np.uint32))


@pytest.mark.parametrize("kind", ["direct", "path", "point"])
def test_oracle_stream_render_equals_reference_render(oracle, kind):
    g = load_golden("render_bf")
    tris, lights = scene(kind)
    img, dims, rng = stream(oracle, kind)
    got = oracle.render_stream(tris, g["r2c"], g["c2w"], XRES, YRES, lights, integrator(kind), img, dims, rng,
                               max_depth=MAX_DEPTH)
    want = g[f"image_{kind}"]
    assert want.mean() > 0.005
    assert rmse(got, want) <= RMSE_TOL
    if kind != "path":
        np.testing.assert_array_equal(got, want)


def gpu_lights(lights):
    out = []
    for lt in lights:
        if lt["type"] == "point":
            out.append(R.point_light(lt["pos"], lt["I"]))
        else:
            out.append(R.mesh_light(lt["first"], lt["ntri"], lt["L"], lt["nsamples"]))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("accel", ["naive", "ray-bvh", "rayhierarchy"])
@pytest.mark.parametrize("kind", ["direct", "path", "point"])
def test_gpu_stream_render_equals_reference_render(gpu_lib, oracle, accel, kind):
    """The GPU wavefront with the reference's sample stream reproduces pbrt's
    breadth-first image (RMSE <= 1e-4; exact for direct lighting) and equals
    the oracle's render of the same stream bit for bit."""
    g = load_golden("render_bf")
    tris, lights = scene(kind)
    img, dims, rng = stream(oracle, kind)
    acc = A.MakeAccelerator(accel, tris)
    cam = R.camera_struct(g["r2c"], g["c2w"], XRES, YRES)
    prm = R.render_params(integrator(kind), spp=SPP, jitter=True, max_depth=MAX_DEPTH)
    got, st = R.render_stream(acc, cam, gpu_lights(lights), prm, img, dims, rng)
    acc.close()
    want = g[f"image_{kind}"]
    assert st["camera_rays"] == XRES * YRES * SPP[0] * SPP[1]
    assert rmse(got, want) <= RMSE_TOL
    if kind != "path":
        np.testing.assert_array_equal(got, want)
    else:
        assert st["bounces"] >= 4
    mine = oracle.render_stream(tris, g["r2c"], g["c2w"], XRES, YRES, lights, integrator(kind), img, dims, rng,
                                max_depth=MAX_DEPTH)
    np.testing.assert_array_equal(got, mine)


@pytest.mark.gpu
def test_gpu_stream_rejects_short_streams(gpu_lib, oracle):
    """A stream whose RNG draws run out, or whose values are fewer than its
    layout needs, is refused with PBG_ERR_INVALID_ARGUMENT."""
    from pbrt_gb300 import _lib as L
    g = load_golden("render_bf")
    tris, lights = scene("path")
    img, dims, rng = stream(oracle, "path")
    acc = A.MakeAccelerator("ray-bvh", tris)
    cam = R.camera_struct(g["r2c"], g["c2w"], XRES, YRES)
    prm = R.render_params("path", spp=SPP, jitter=True, max_depth=MAX_DEPTH)
    with pytest.raises(L.PbgError) as e:
        R.render_stream(acc, cam, gpu_lights(lights), prm, img, dims, rng[:100])
    assert e.value.status == L.PBG_ERR_INVALID_ARGUMENT
    with pytest.raises(L.PbgError) as e:
        R.render_stream(acc, cam, gpu_lights(lights), prm, img, dims[:, :12], rng)
    assert e.value.status == L.PBG_ERR_INVALID_ARGUMENT
    acc.close()
