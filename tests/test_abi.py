"""The C-ABI library builds, loads without a GPU and exports every function
declared in include/cs_gb300.h; the Python binding declares each of them."""
import os
import re

from conftest import ROOT, pkg


def _declared():
    src = open(os.path.join(ROOT, "include", "cs_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cs_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    cs = pkg()
    cs.build.build_library()
    lib = cs._lib.load()
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(cs._lib.SIGNATURES) == names


def test_errors_are_codes_not_exceptions():
    import ctypes
    cs = pkg()
    lib = cs._lib.load()
    out = ctypes.c_void_p()
    rc = lib.cs_module_load(None, ctypes.byref(out))
    assert rc == 1  # CS_ERR_INVALID
    assert "null" in cs._lib.last_error()
