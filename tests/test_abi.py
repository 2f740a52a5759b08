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


def test_noalloc_entry_point_calls_no_allocator():
    """cs_babd_solve_noalloc and the helpers it calls name no device or host
    allocator (its scratch is the library's static device array)."""
    src = open(os.path.join(ROOT, "collocation-solver-cuda_gb300", "csrc", "cs_babd.cu")).read()

    def body(name):
        i = src.index(name + "(")
        j = src.index("{", i)
        depth, k = 0, j
        while True:
            depth += {"{": 1, "}": -1}.get(src[k], 0)
            k += 1
            if depth == 0:
                return src[j:k]

    allocators = re.compile(r"cuda(Malloc|Free|MallocAsync|FreeAsync|MallocManaged|MallocHost|HostAlloc)|\bmalloc\(|"
                            r"\bnew\b|torch|\bcuMem")
    for fn in ("extern \"C\" int cs_babd_solve_noalloc", "int noalloc_scratch", "int babd_run"):
        assert not allocators.search(body(fn)), fn
