"""The learned traversal ordering: tensor-core backward pass against the
float64 oracle, training convergence, and results identical with the
ordering on and off."""
import ctypes as C

import numpy as np
import pytest

from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

pytestmark = pytest.mark.gpu

NPARAM = 64 * 112 + 64 + 64 * 64 + 64 + 256 * 64 + 256


class LearnParams(C.Structure):
    _fields_ = [("batch", C.c_int32), ("steps_per_train", C.c_int32), ("lr", C.c_float),
                ("momentum", C.c_float), ("records", C.c_int32), ("reserved0", C.c_int32),
                ("seed", C.c_uint64), ("reserved", C.c_int32 * 8)]


class LearnStats(C.Structure):
    _fields_ = [("trained_steps", C.c_uint64), ("records", C.c_uint64), ("last_loss", C.c_float),
                ("last_accuracy", C.c_float), ("infer_ms", C.c_double), ("train_ms", C.c_double)]


def bind(lib):
    vp = C.c_void_p
    lib.pbg_learn_enable.argtypes = [vp, C.c_int32, C.POINTER(LearnParams)]
    lib.pbg_learn_train.argtypes = [vp, C.c_int32]
    lib.pbg_learn_get_stats.argtypes = [vp, C.POINTER(LearnStats)]
    lib.pbg_learn_params_io.argtypes = [vp, vp, C.c_int32]
    lib.pbg_learn_gradients.argtypes = [vp, vp, vp, C.c_int32, vp, vp]
    return lib


def small_bvh_scene():
    sc = S.displaced_icospheres(seed=3, n_inst=60, box=16.0)
    return A.MakeAccelerator("ray-bvh", sc["tris"]), sc["tris"]


def test_backward_matches_float64_oracle(gpu_lib):
    from oracle import mlp_oracle as M
    lib = bind(gpu_lib.lib())
    acc, _ = small_bvh_scene()
    p = LearnParams()
    p.seed = 7
    assert lib.pbg_learn_enable(acc.handle, 1, C.byref(p)) == 0, gpu_lib.last_error()
    params = np.empty(NPARAM, np.float32)
    assert lib.pbg_learn_params_io(acc.handle, params.ctypes.data, 1) == 0
    g = np.random.default_rng(3)
    B = 256
    x = g.normal(size=(B, 112)).astype(np.float32)
    x[:, 105:] = 0
    y = g.integers(0, 256, size=B).astype(np.int32)
    grads = np.empty(NPARAM, np.float32)
    loss = C.c_float()
    rc = lib.pbg_learn_gradients(acc.handle, x.ctypes.data, y.ctypes.data, B, grads.ctypes.data,
                                 C.byref(loss))
    assert rc == 0, gpu_lib.last_error()
    want, wloss = M.gradients(params, x, y)
    assert abs(loss.value - wloss) <= 1e-3 * max(1.0, abs(wloss))
    k = 0
    for name, n in zip(["W1", "b1", "W2", "b2", "W3", "b3"], M.SIZES):
        a, b = grads[k:k + n].astype(np.float64), want[k:k + n]
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-12)
        assert err < 2e-2, f"{name}: relative error {err}"
        k += n


def test_training_reduces_loss_and_results_unchanged(gpu_lib, oracle):
    lib = bind(gpu_lib.lib())
    acc, tris = small_bvh_scene()
    rays = S.random_rays(65536, -8.0, 8.0, seed=31)
    plain = acc.Intersect(rays.copy())
    plain_occ = acc.IntersectP(rays)
    p = LearnParams()
    p.batch = 4096
    p.steps_per_train = 40
    p.lr = 0.1
    assert lib.pbg_learn_enable(acc.handle, 1, C.byref(p)) == 0, gpu_lib.last_error()
    st = LearnStats()
    losses = []
    for rnd in range(4):  # collect records from nearest-hit batches, then train
        acc.Intersect(S.random_rays(65536, -8.0, 8.0, seed=100 + rnd).copy())
        assert lib.pbg_learn_train(acc.handle, 0) == 0, gpu_lib.last_error()
        assert lib.pbg_learn_get_stats(acc.handle, C.byref(st)) == 0
        losses.append(st.last_loss)
    assert st.trained_steps > 0 and st.records > 0
    assert losses[-1] < losses[0], losses
    # ordered traversal: identical hits and occlusion
    ordered = acc.Intersect(rays.copy())
    for a, b in zip(ordered, plain):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(acc.IntersectP(rays), plain_occ)
    want = oracle.BVH(tris).nearest(rays)
    np.testing.assert_array_equal(ordered[0], want[0])
