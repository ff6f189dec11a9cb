"""The C ABI library loads and exports every function that include/chiml_gpu.h declares."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    txt = open(os.path.join(ROOT, "include", "chiml_gpu.h")).read()
    return sorted(set(re.findall(r"\b(chiml_[a-z_]+)\s*\(", txt)))


def test_header_symbols_exported(built_engine):
    lib = ctypes.CDLL(built_engine)
    names = _declared()
    assert "chiml_create" in names and "chiml_step" in names
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from chiml_gb300 import api
    assert set(_declared()) == set(api.EXPORTED)


def test_missing_library_fails_loudly(tmp_path):
    from chiml_gb300 import api
    try:
        api.load_library(str(tmp_path / "nope.so"))
    except FileNotFoundError:
        return
    raise AssertionError("no error for a missing engine library")
