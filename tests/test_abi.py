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


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of chiml_stats and chiml_options have the C structs' size and field
    offsets (a mismatch would make chiml_query misread every field after it)."""
    import shutil
    import subprocess
    import pytest
    from chiml_gb300 import api
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    checks = {"chiml_stats": api.Stats, "chiml_options": api._Options}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "chiml_gpu.h"', "int main(void) {"]
    for cname, py in checks.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in checks.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
