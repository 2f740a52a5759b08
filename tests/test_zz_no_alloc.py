"""cs_babd_solve_noalloc: the BABD solve for callers that cannot allocate
device memory (inside an allocator or memory pool they must not re-enter, or
under a framework that owns all device memory).  It must give the results of
cs_babd_solve, call after call on the one shared scratch array, and refuse
systems larger than that array.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden, pkg

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _solve(lib, fn, ny, npar, n, system):
    A, C, H, b, B0, Bn, Vn, r = system
    ins = [_dev(x) for x in (A, C, H if npar else np.zeros(1), b, B0, Bn, Vn if npar else np.zeros(1), r)]
    dy = torch.zeros((n + 1) * ny, dtype=torch.float64, device="cuda")
    dp = torch.zeros(max(npar, 1), dtype=torch.float64, device="cuda")
    sing = ctypes.c_int(-1)
    torch.cuda.synchronize()
    rc = getattr(lib, fn)(ny, npar, n, *[ctypes.c_void_p(t.data_ptr()) for t in ins], ctypes.c_void_p(dy.data_ptr()),
                          ctypes.c_void_p(dp.data_ptr()), ctypes.byref(sing), None)
    torch.cuda.synchronize()
    return rc, dy.cpu().numpy().reshape(n + 1, ny), dp.cpu().numpy()[:npar], sing.value


def _random_system(ny, npar, n, seed):
    rng = np.random.default_rng(seed)
    A = -np.eye(ny)[None] + 0.2 * rng.standard_normal((n, ny, ny))
    C = np.broadcast_to(np.eye(ny), (n, ny, ny)).copy()
    H = 0.1 * rng.standard_normal((n, ny, npar))
    b = rng.standard_normal((n, ny))
    return (A, C, H, b, rng.standard_normal((ny + npar, ny)), rng.standard_normal((ny + npar, ny)),
            rng.standard_normal((ny + npar, npar)), rng.standard_normal(ny + npar))


def test_noalloc_matches_allocating_solve_on_consecutive_calls():
    cs = pkg()
    lib = cs._lib.load()
    g = golden("stage_vdp_n21_m4")
    ny, npar, n = int(g["ny"]), int(g["np"]), int(g["N"]) - 1
    first = (g["A"].reshape(n, ny, ny), g["C"].reshape(n, ny, ny), g["H"].reshape(n, ny, npar), g["b"],
             g["B_0"], g["B_n"], g["V_n"], g["r_bc"])
    second = _random_system(5, 3, 300, seed=11)
    # two calls in a row on the shared scratch: a small system, then a larger
    # one with other sizes, each against the allocating entry point
    for (ny_, np_, n_), system in (((ny, npar, n), first), ((5, 3, 300), second)):
        rc0, dy0, dp0, s0 = _solve(lib, "cs_babd_solve", ny_, np_, n_, system)
        rc1, dy1, dp1, s1 = _solve(lib, "cs_babd_solve_noalloc", ny_, np_, n_, system)
        assert rc0 == 0 and rc1 == 0, cs._lib.last_error()
        assert s0 == s1 == 0
        scale = max(1.0, np.abs(dy0).max())
        np.testing.assert_allclose(dy1, dy0, rtol=0, atol=1e-8 * scale)
        np.testing.assert_allclose(dp1, dp0, rtol=0, atol=1e-8 * scale)
    # and the first system again, after the larger one left its data behind
    rc0, dy0, dp0, _ = _solve(lib, "cs_babd_solve", ny, npar, n, first)
    rc1, dy1, dp1, _ = _solve(lib, "cs_babd_solve_noalloc", ny, npar, n, first)
    assert rc0 == 0 and rc1 == 0
    np.testing.assert_allclose(dy1, dy0, rtol=0, atol=1e-8 * max(1.0, np.abs(dy0).max()))
    np.testing.assert_allclose(dy1, g["delta_y"], rtol=0, atol=1e-8 * max(1.0, np.abs(g["delta_y"]).max()))


def test_noalloc_without_parameters():
    """np = 0 with H, Vn and dp passed as NULL, which the entry point
    accepts: same solution as the allocating solve."""
    cs = pkg()
    lib = cs._lib.load()
    ny, n = 6, 257
    A, C, _, b, B0, Bn, _, r = _random_system(ny, 0, n, seed=5)
    ins = [_dev(x) for x in (A, C, b, B0, Bn, r)]
    outs = []
    for fn in ("cs_babd_solve", "cs_babd_solve_noalloc"):
        dy = torch.zeros((n + 1) * ny, dtype=torch.float64, device="cuda")
        sing = ctypes.c_int(-1)
        torch.cuda.synchronize()
        a, c, bb, b0, bn, rr = [ctypes.c_void_p(t.data_ptr()) for t in ins]
        rc = getattr(lib, fn)(ny, 0, n, a, c, None, bb, b0, bn, None, rr, ctypes.c_void_p(dy.data_ptr()), None,
                              ctypes.byref(sing), None)
        torch.cuda.synchronize()
        assert rc == 0, cs._lib.last_error()
        assert sing.value == 0
        outs.append(dy.cpu().numpy())
    np.testing.assert_allclose(outs[1], outs[0], rtol=0, atol=1e-8 * max(1.0, np.abs(outs[0]).max()))


def test_noalloc_leaves_free_device_memory_unchanged():
    """A call near the size limit (ny = 4, np = 2: 25,000 intervals, where the
    allocating solve takes about 30 MB) changes the free device memory by
    nothing once the library is loaded."""
    cs = pkg()
    lib = cs._lib.load()
    ny, npar, n = 4, 2, 25000
    system = _random_system(ny, npar, n, seed=9)
    rc, dy0, _, _ = _solve(lib, "cs_babd_solve_noalloc", ny, npar, n, system)  # loads the library's module
    assert rc == 0, cs._lib.last_error()
    A, C, H, b, B0, Bn, Vn, r = [_dev(x) for x in system]
    dy = torch.zeros((n + 1) * ny, dtype=torch.float64, device="cuda")
    dp = torch.zeros(npar, dtype=torch.float64, device="cuda")
    sing = ctypes.c_int(-1)
    args = [ctypes.c_void_p(t.data_ptr()) for t in (A, C, H, b, B0, Bn, Vn, r, dy, dp)]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = lib.cs_babd_solve_noalloc(ny, npar, n, *args, ctypes.byref(sing), None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == 0, cs._lib.last_error()
    assert free1 == free0
    np.testing.assert_array_equal(dy.cpu().numpy().reshape(n + 1, ny), dy0)


def test_noalloc_rejects_systems_beyond_its_scratch():
    cs = pkg()
    lib = cs._lib.load()
    # ny = 4, np = 2 needs 148 doubles per interval: 30000 intervals exceed 32 MiB
    one = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(one.data_ptr())
    rc = lib.cs_babd_solve_noalloc(4, 2, 30000, *([p] * 10), None, None)
    assert rc == 1  # CS_ERR_INVALID, nothing launched
    msg = cs._lib.last_error()
    assert "scratch" in msg and "cs_babd_solve" in msg
