"""The tcgen05 BF16 GEMM (the learned ordering's tensor-core building block)
against a float64 product of the same BF16 values."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    """float32 -> bf16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bf16_bits(h):
    return (h.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("M,N,K,acc", [(128, 16, 16, 0), (256, 64, 112, 0), (128, 256, 128, 0),
                                       (384, 64, 304, 0), (256, 128, 64, 1)])
def test_tc_gemm_matches_float64(gpu_lib, M, N, K, acc):
    torch = pytest.importorskip("torch")
    lib = gpu_lib.lib()
    fn = lib.pbg_tc_gemm_bf16
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                   C.c_void_p]
    g = np.random.default_rng(M * 7 + N * 3 + K)
    a = to_bf16_bits(g.normal(size=(M, K)))
    b = to_bf16_bits(g.normal(size=(N, K)))
    c0 = g.normal(size=(M, N)).astype(np.float32)
    da = torch.from_numpy(a.view(np.int16)).cuda()
    db = torch.from_numpy(b.view(np.int16)).cuda()
    dc = torch.from_numpy(c0.copy()).cuda()
    rc = fn(da.data_ptr(), db.data_ptr(), dc.data_ptr(), M, N, K, acc, None)
    assert rc == 0, gpu_lib.last_error()
    got = dc.cpu().numpy()
    want = from_bf16_bits(a).astype(np.float64) @ from_bf16_bits(b).astype(np.float64).T
    if acc:
        want = want + c0
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4 * np.abs(want).max())
