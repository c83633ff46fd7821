import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import pbg_import  # noqa: E402

pbg_import.load()

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


GOLDEN_CASES = ["sphere_small", "grid_ties", "degenerate", "soup", "limits", "empty"]


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    import pbrt_gb300._lib as L
    if not os.path.exists(L.LIB_PATH):
        L.build()
    lib = L.lib()
    if lib.pbg_device_count() == 0:
        pytest.fail("no CUDA device visible: the gpu tests need a GB300")
    return L
