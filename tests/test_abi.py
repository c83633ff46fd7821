"""The C ABI library loads and exports every entry point its header
declares; no device work is issued here."""
import ctypes

import pbrt_gb300._lib as L


def test_library_exports_every_declared_symbol():
    lib = L.lib()
    names = L.exported_symbols_in_header()
    assert "pbg_intersect" in names and "pbg_occluded" in names
    for name in names:
        assert hasattr(lib, name), name
        assert isinstance(getattr(lib, name), ctypes._CFuncPtr)


def test_version_and_status_strings():
    lib = L.lib()
    assert b"sm_103a" in lib.pbg_version()
    for code in range(8):
        assert L.status_string(code)
    assert L.status_string(99) == "unknown status"


def test_invalid_arguments_return_status_not_abort():
    lib = L.lib()
    assert lib.pbg_scene_create(None, None, 4, 0, None, None) == L.PBG_ERR_INVALID_ARGUMENT
    out = ctypes.c_void_p()
    assert lib.pbg_scene_create(None, None, 0, 42, None, ctypes.byref(out)) == L.PBG_ERR_INVALID_ARGUMENT
    assert lib.pbg_intersect(None, None, 1, None) == L.PBG_ERR_INVALID_ARGUMENT
    assert lib.pbg_occluded(None, None, 1, None) == L.PBG_ERR_INVALID_ARGUMENT
    assert lib.pbg_stats(None, None) == L.PBG_ERR_INVALID_ARGUMENT
    assert "bad" in L.last_error() or L.last_error() != ""


def test_make_accelerator_names():
    import pytest
    from pbrt_gb300 import accel as A
    with pytest.raises(ValueError):
        A.MakeAccelerator("kdtree", [[0, 0, 0, 1, 0, 0, 0, 1, 0]])


def test_struct_mirrors_match_the_header(tmp_path):
    """Every ctypes mirror of a header struct has the header's size and, field
    by field, the header's offsets (a C program compiled by gcc against
    include/pbrt_gb300.h prints them)."""
    import shutil
    import subprocess
    from pathlib import Path

    import pytest
    from pbrt_gb300 import batch as Bt
    from pbrt_gb300 import render as R
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    mirrors = {"pbg_params": L.Params, "pbg_rays": L.Rays, "pbg_hits": L.Hits, "pbg_counters": L.Counters,
               "pbg_learn_params": L.LearnParams, "pbg_learn_stats": L.LearnStats,
               "pbg_batch_params": Bt.BatchParams, "pbg_batch_stats": Bt.BatchStats,
               "pbg_camera": R.Camera, "pbg_light": R.Light, "pbg_render_params": R.RenderParams,
               "pbg_render_stats": R.RenderStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "pbrt_gb300.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'printf("{cname} :size %zu\\n", sizeof({cname}));')
        for name, *_ in cls._fields_:
            lines.append(f'printf("{cname} {name} %zu\\n", offsetof({cname}, {name}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parents[1] / "include"
    subprocess.run(["gcc", "-std=c11", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, name, value = line.split()
        got[(cname, name)] = int(value)
    for cname, cls in mirrors.items():
        assert got[(cname, ":size")] == ctypes.sizeof(cls), cname
        for name, *_ in cls._fields_:
            assert got[(cname, name)] == getattr(cls, name).offset, (cname, name)


def test_noalloc_rejects_misaligned_views():
    """The allocation-free entry point reads rays as float4 and the rest as
    4-byte words: a misaligned view is refused with a status before any
    device work (the pointers here are never dereferenced)."""
    lib = L.lib()
    fn = lib.pbg_intersect_naive_noalloc
    vp = ctypes.c_void_p
    fn.argtypes = [vp, ctypes.c_int64, vp, vp, ctypes.c_int64, vp, vp, vp, vp, vp]
    a, odd8, odd2 = vp(1 << 16), vp((1 << 16) + 8), vp((1 << 16) + 2)
    assert fn(a, 1, odd8, a, 1, a, a, a, a, None) == L.PBG_ERR_INVALID_ARGUMENT
    assert "16-byte" in L.last_error()
    assert fn(a, 1, a, odd8, 1, a, a, a, a, None) == L.PBG_ERR_INVALID_ARGUMENT
    assert fn(odd2, 1, a, a, 1, a, a, a, a, None) == L.PBG_ERR_INVALID_ARGUMENT
    assert fn(a, 1, a, a, 1, a, odd2, a, a, None) == L.PBG_ERR_INVALID_ARGUMENT
