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
