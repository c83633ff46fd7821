"""pbrt's Cross() component, (float)((double)a*b - (double)c*d), restated in
FP32 error-free arithmetic (pbrt-v2_gb300/csrc/pbg_xcross.h): every result the
FP32 form claims must equal the double form bit for bit, and generic inputs
must almost never need the FP64 fallback.  Host build of the same header the
kernels include."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("xcross") / "xcross_check")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                           os.path.join(HERE, "native", "xcross_check.cpp")])
    return exe


def test_proven_results_equal_double_form(checker):
    out = subprocess.run([checker, "20000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    n, proven, fallback, bad = map(int, out.stdout.split()[-4:])
    assert bad == 0
    assert proven + fallback == n
    # six of the eight input families are adversarial (cancellation,
    # midpoints, specials, out-of-range magnitudes); the rest never fall back
    assert proven > n // 2
