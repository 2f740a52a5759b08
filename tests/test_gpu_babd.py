"""cs_babd_solve (standalone BABD solve, device pointers) against the
reference's partitioned solve: the golden per-stage dumps and the oracle on
larger random systems.  Tolerance: 1e-8 relative to the solution's scale."""
import ctypes

import numpy as np
import pytest

from conftest import golden, pkg
from oracle import collocation_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def babd_gpu(cs, fn, ny, npar, n, A, C, H, b, B0, Bn, Vn, r):
    lib = cs._lib.load()
    ins = [_dev(x) for x in (A, C, H if npar else np.zeros(1), b, B0, Bn, Vn if npar else np.zeros(1), r)]
    dy = torch.zeros((n + 1) * ny, dtype=torch.float64, device="cuda")
    dp = torch.zeros(max(npar, 1), dtype=torch.float64, device="cuda")
    sing = ctypes.c_int(-1)
    torch.cuda.synchronize()
    rc = getattr(lib, fn)(ny, npar, n, *[ctypes.c_void_p(t.data_ptr()) for t in ins], ctypes.c_void_p(dy.data_ptr()),
                          ctypes.c_void_p(dp.data_ptr()), ctypes.byref(sing), None)
    cs._lib.check(rc, fn)
    torch.cuda.synchronize()
    return dy.cpu().numpy().reshape(n + 1, ny), dp.cpu().numpy()[:npar], sing.value


def random_babd(ny, npar, n, seed):
    """A well-conditioned random system with the structure the condensation
    produces (C = I, A = -I + small)."""
    rng = np.random.default_rng(seed)
    A = -np.eye(ny)[None] + 0.2 * rng.standard_normal((n, ny, ny))
    C = np.broadcast_to(np.eye(ny), (n, ny, ny)).copy()
    H = 0.1 * rng.standard_normal((n, ny, npar))
    b = rng.standard_normal((n, ny))
    B0 = rng.standard_normal((ny + npar, ny))
    Bn = rng.standard_normal((ny + npar, ny))
    Vn = rng.standard_normal((ny + npar, npar))
    r = rng.standard_normal(ny + npar)
    return A, C, H, b, B0, Bn, Vn, r


@pytest.mark.parametrize("case", ["vdp_n21_m4", "dint_n33_m3", "pend2_n21_m5", "econ_n17_m3"])
def test_babd_solve_matches_reference(case):
    cs = pkg()
    g = golden("stage_" + case)
    ny, npar, N = int(g["ny"]), int(g["np"]), int(g["N"])
    n = N - 1
    dy, dp, sing = babd_gpu(cs, "cs_babd_solve", ny, npar, n, g["A"].reshape(n, ny, ny), g["C"].reshape(n, ny, ny),
                            g["H"].reshape(n, ny, npar), g["b"], g["B_0"], g["B_n"], g["V_n"], g["r_bc"])
    assert sing == 0
    scale = max(1.0, np.abs(g["delta_y"]).max())
    np.testing.assert_allclose(dy, g["delta_y"], rtol=0, atol=1e-8 * scale)
    np.testing.assert_allclose(dp, g["delta_p"], rtol=0, atol=1e-8 * scale)


@pytest.mark.parametrize("ny,npar,n", [(4, 2, 1000), (8, 0, 777), (5, 3, 65)])
def test_babd_solve_matches_oracle(ny, npar, n):
    cs = pkg()
    A, C, H, b, B0, Bn, Vn, r = random_babd(ny, npar, n, seed=ny * 100 + n)
    dy, dp, sing = babd_gpu(cs, "cs_babd_solve", ny, npar, n, A, C, H, b, B0, Bn, Vn, r)
    ref_dy, ref_dp = O.solve_babd(ny, npar, n + 1, A.reshape(-1, ny), C.reshape(-1, ny), H.reshape(n * ny, npar), b,
                                  B0, Bn, Vn, r)
    assert sing == 0
    scale = max(1.0, np.abs(ref_dy).max())
    np.testing.assert_allclose(dy, ref_dy, rtol=0, atol=1e-8 * scale)
    np.testing.assert_allclose(dp, ref_dp, rtol=0, atol=1e-8 * scale)


def test_babd_solve_rejects_bad_sizes():
    cs = pkg()
    lib = cs._lib.load()
    nul = [None] * 10
    assert lib.cs_babd_solve(40, 0, 10, *nul, None, None) == 1
    assert "ny" in cs._lib.last_error()


@pytest.mark.parametrize("fn", ["cs_babd_solve", "cs_babd_solve_noalloc"])
@pytest.mark.parametrize("scale", [1e-9, 1e9])
def test_babd_solve_is_scale_invariant(fn, scale):
    """Every equation multiplied by the same factor leaves the solution
    unchanged: no reflection may be skipped because its column is small in
    absolute terms (a system scaled by 1e-9 has columns of norm ~1e-9)."""
    cs = pkg()
    ny, npar, n = 4, 2, 300
    A, C, H, b, B0, Bn, Vn, r = random_babd(ny, npar, n, seed=77)
    dy0, dp0, s0 = babd_gpu(cs, fn, ny, npar, n, A, C, H, b, B0, Bn, Vn, r)
    dy1, dp1, s1 = babd_gpu(cs, fn, ny, npar, n, *[scale * x for x in (A, C, H, b, B0, Bn, Vn, r)])
    assert s0 == s1 == 0
    sc = max(1.0, np.abs(dy0).max())
    np.testing.assert_allclose(dy1, dy0, rtol=0, atol=1e-10 * sc)
    np.testing.assert_allclose(dp1, dp0, rtol=0, atol=1e-10 * sc)
