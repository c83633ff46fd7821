"""Registers the in-tree package directory ``pbrt-v2_gb300/`` under the
importable name ``pbrt_gb300`` (the directory name is not an identifier)."""
import importlib.util
import os
import sys

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "pbrt-v2_gb300")


def load():
    if "pbrt_gb300" in sys.modules:
        return sys.modules["pbrt_gb300"]
    spec = importlib.util.spec_from_file_location(
        "pbrt_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["pbrt_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod
