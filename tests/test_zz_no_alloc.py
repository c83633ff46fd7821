"""The allocation-free nearest-hit entry point, for callers that cannot call
cudaMalloc (an allocator-hooked host, a fully committed device), against
the regular naive scene path: identical hits on two calls in a row.

Kept in its own file, collected last, so that a failure here comes after
every other test has run."""
import ctypes as C

import numpy as np
import pytest

from pbrt_gb300 import accel as A
from pbrt_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _dev_rays(torch, rays):
    o = torch.from_numpy(np.ascontiguousarray(np.stack([rays[0], rays[1], rays[2], rays[6]], 1))).cuda()
    d = torch.from_numpy(np.ascontiguousarray(np.stack([rays[3], rays[4], rays[5], rays[7]], 1))).cuda()
    return o, d


def test_noalloc_matches_scene_path_two_calls(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib.lib()
    fn = lib.pbg_intersect_naive_noalloc
    vp = C.c_void_p
    fn.argtypes = [vp, C.c_int64, vp, vp, C.c_int64, vp, vp, vp, vp, vp]
    cfg = S.config_small_naive()
    tris = cfg["tris"]
    tri_dev = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
    acc = A.MakeAccelerator("naive", tris)
    batches = [cfg["rays"], S.random_rays(40000, -3.0, 3.0, seed=21)]
    batches[1][7, ::3] = 2.5  # finite maxt on a third of the rays
    for rays in batches:  # two calls in a row share the fixed scratch
        n = rays.shape[1]
        o, d = _dev_rays(torch, rays)
        outs = [torch.empty(n, dtype=torch.int32, device="cuda")] + \
               [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3)]
        ref = [torch.empty(n, dtype=torch.int32, device="cuda")] + \
              [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3)]
        st = torch.cuda.current_stream().cuda_stream
        rc = fn(tri_dev.data_ptr(), len(tris), o.data_ptr(), d.data_ptr(), n,
                *[x.data_ptr() for x in outs], st)
        assert rc == 0, gpu_lib.last_error()
        acc.intersect_device(o, d, *ref, stream=torch.cuda.current_stream())
        torch.cuda.synchronize()
        got = [x.cpu().numpy() for x in outs]
        want = [x.cpu().numpy() for x in ref]
        np.testing.assert_array_equal(got[0], want[0])
        h = want[0] >= 0
        assert h.any()
        for k in (1, 2, 3):
            np.testing.assert_array_equal(got[k][h], want[k][h])


def test_noalloc_rejects_oversized_batch(gpu_lib):
    lib = gpu_lib.lib()
    fn = lib.pbg_intersect_naive_noalloc
    vp = C.c_void_p
    fn.argtypes = [vp, C.c_int64, vp, vp, C.c_int64, vp, vp, vp, vp, vp]
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = fn(dummy, 1, dummy, dummy, (1 << 20) + 1, dummy, dummy, dummy, dummy, None)
    assert rc == gpu_lib.PBG_ERR_INVALID_ARGUMENT
    assert "1048576" in gpu_lib.last_error()
