"""Pin the oracle (CPU restatement, oracle/collocation_oracle.py) and the
collocation tables against golden vectors produced by running the unmodified
reference (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden, oracle_problem, pkg
from oracle import collocation_oracle as O

STAGES = [("vdp_n21_m4", "vdp"), ("vdp_n33_m5", "vdp"), ("dint_n33_m3", "dint_param"),
          ("pend2_n21_m5", "pend2"), ("econ_n17_m3", "eqcon")]
E2E = [("vdp_cfg1", "vdp"), ("vdp_coarse", "vdp_coarse"), ("dint_param", "dint_param"), ("vdp_input", "vdp_input"),
       ("pend2", "pend2"), ("vdp_ineq", "vdp_ineq"), ("vdp_svineq", "vdp_svineq"), ("vdp_m7", "vdp"),
       ("eqcon", "eqcon")]


def test_lobatto_and_gauss_tables_match_reference():
    cs = pkg()
    g = golden("tables")
    for m in range(3, 10):
        lo = cs.tables.lobatto(m)
        tol = 1e-14 if m <= 6 else 5e-12
        np.testing.assert_allclose(lo.A, g["A%d" % m], atol=tol)
        np.testing.assert_allclose(lo.b, g["b%d" % m], atol=tol)
        np.testing.assert_allclose(lo.c, g["c%d" % m], atol=1e-15)
        st = cs.tables.segment_tables(m)
        np.testing.assert_allclose(st["L"], g["L%d" % m], atol=1e-12)
        np.testing.assert_allclose(st["I"], g["I%d" % m], atol=1e-10)
    # m = 10: the reference's table leaves A[8, 0] unset (0.0); every other
    # entry agrees with the exact tableau
    lo, ref = cs.tables.lobatto(10), g["A10"]
    diff = np.abs(lo.A - ref)
    assert ref[8, 0] == 0.0 and lo.A[8, 0] > 0.01
    diff[8, 0] = 0.0
    assert diff.max() < 1e-10
    for n in range(2, 12):
        ga = cs.tables.gauss(n)
        tol = 1e-15 if n < 11 else 1e-10  # the reference's 11-point nodes carry 11 digits
        np.testing.assert_allclose(ga.t, g["gt%d" % n], atol=max(tol, 4e-16))
        np.testing.assert_allclose(ga.w, g["gw%d" % n], atol=1e-15)


def test_lobatto_order_conditions():
    cs = pkg()
    for m in range(3, 11):
        lo = cs.tables.lobatto(m)
        np.testing.assert_allclose(lo.A.sum(axis=1), lo.c, atol=1e-14)
        for q in range(1, 2 * m - 2):  # b integrates polynomials of degree 2m-3
            np.testing.assert_allclose(np.dot(lo.b, lo.c ** (q - 1)), 1.0 / q, atol=1e-13)


@pytest.mark.parametrize("case,prob", STAGES)
def test_oracle_stages_match_reference(case, prob):
    cs = pkg()
    g = golden("stage_" + case)
    P = oracle_problem(prob)
    m, N = int(g["m"]), int(g["N"])
    ny, nz, npar = P.ny, P.nz, P.np
    rk, seg = cs.tables.lobatto(m), cs.tables.segment_tables(m)
    t, p, alpha, tol = g["t"], g["p"], float(g["alpha"]), float(g["tol"])
    close = dict(rtol=1e-11, atol=1e-11)

    y, yd0, zt0 = O.form_initial_input(P, m, N, g["y0"], g["z0"], p, rk)
    np.testing.assert_allclose(yd0, g["init_y_dot"], **close)
    np.testing.assert_allclose(zt0, g["init_z_tilde"], **close)

    y, yd, zt = g["y"], g["y_dot"], g["z_tilde"]
    f_q, y_tilde, f_a, f_b, r_bc = O.compute_f_q(P, m, N, rk, t, y, yd, zt, p, alpha)
    for k, v in dict(f_q=f_q, y_tilde=y_tilde, f_a=f_a, f_b=f_b, r_bc=r_bc).items():
        np.testing.assert_allclose(v, g[k], err_msg=k, **close)

    J, V, D, W, B0, Bn, Vn = O.construct_jacobian(P, m, N, rk, t, y, y_tilde, zt, p, alpha)
    for k, v in dict(J=J, V=V, D=D, W=W, B_0=B0, B_n=Bn, V_n=Vn).items():
        np.testing.assert_allclose(v, g[k], err_msg=k, **close)

    A, C, H, b = O.reduce_jacobian(ny, nz, npar, m, N, W, D, J, V, f_a, f_b)
    for k, v in dict(A=A, C=C, H=H, b=b).items():
        np.testing.assert_allclose(v, g[k], err_msg=k, rtol=1e-9, atol=1e-9)

    # partitioned BABD factorisation: reference inputs, element-wise outputs
    idx, R, E, Jr, G, d, At, Ct, Ht, bt = O.partition_factorization(ny, npar, 8, N, g["A"], g["C"], g["H"], g["b"])
    np.testing.assert_array_equal(idx, g["index"])
    for k, v in dict(R=R, E=E, J_red=Jr, G=G, d=d, A_tilde=At, C_tilde=Ct, H_tilde=Ht, b_tilde=bt).items():
        ref = g[k]
        # rows of the last interval of each partition are never written by the
        # reference (its device arrays start as NaN here): compare written rows
        ok = np.isfinite(ref)
        assert ok.mean() >= 0.5
        np.testing.assert_allclose(v[ok], ref[ok], err_msg=k, rtol=1e-9, atol=1e-9)

    ds_r, dp = O.reduced_babd_solve(ny, npar, 8, g["A_tilde"], g["C_tilde"], g["H_tilde"], g["b_tilde"],
                                    g["B_0"], g["B_n"], g["V_n"], -g["r_bc"])
    np.testing.assert_allclose(ds_r, g["delta_s_r"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(dp, g["delta_p"], rtol=1e-8, atol=1e-8)
    dy = O.partition_backward_substitution(ny, npar, 8, N, g["index"], g["delta_s_r"], g["delta_p"],
                                           g["R"], g["G"], g["E"], g["J_red"], g["d"])
    np.testing.assert_allclose(dy, g["delta_y"], rtol=1e-8, atol=1e-8)
    dk, dyd, dzt = O.recover_delta_k(ny, nz, m, N, g["delta_y"], g["delta_p"], g["f_a"], g["J"], g["V"], g["W"])
    np.testing.assert_allclose(dk, g["delta_k"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(dyd, g["delta_y_dot"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(dzt, g["delta_z_tilde"], rtol=1e-8, atol=1e-8)

    res, mx = O.segment_residual(P, m, N, t, y, yd, zt, p, alpha, tol, seg)
    np.testing.assert_allclose(res, g["seg_residual"], rtol=1e-10, atol=1e-12)
    assert abs(mx - float(g["seg_max"])) <= 1e-10 * abs(mx)

    z = O.recover_solution(nz, m, N, zt, seg)
    np.testing.assert_allclose(z, g["z_nodes"], rtol=1e-13, atol=1e-13)

    Nn, tn, yn, zn = O.remesh(ny, nz, N, t, y, g["z_nodes"], g["remesh_residual"])
    assert Nn == int(g["remesh_N"])
    np.testing.assert_array_equal(tn, g["remesh_t"])
    np.testing.assert_array_equal(yn, g["remesh_y"])
    np.testing.assert_array_equal(zn, g["remesh_z"])


@pytest.mark.parametrize("case,prob", E2E)
def test_oracle_end_to_end_matches_reference(case, prob):
    cs = pkg()
    g = golden("e2e_" + case)
    P = oracle_problem(prob)
    m = int(g["m"])
    r = O.solve(P, m, cs.tables.lobatto(m), cs.tables.segment_tables(m))
    assert r.success == bool(g["success"])
    assert r.N == g["t"].shape[0]
    assert r.jacobian_count == int(g["jacobian_counts"])
    assert r.residual_count == int(g["residual_counts"])
    assert r.nodes_after_remesh == list(g["nodes_after_remesh"])
    # the reference prints the norms with 8 decimals
    np.testing.assert_array_equal(np.round(np.array(r.norms), 8), g["norms"])
    np.testing.assert_array_equal(r.t, g["t"])
    # 1e-8 of each array's scale (a state constraint's multiplier reaches ~300)
    for k, got in (("y", r.y), ("z", r.z), ("p", r.p)):
        np.testing.assert_allclose(got, g[k], atol=1e-8 * max(1.0, np.abs(g[k]).max(initial=0.0)), rtol=0)


MODES = [(rt, sc) for rt in (0, 1, 2) for sc in (True, False)]


@pytest.mark.parametrize("case,prob", STAGES)
def test_oracle_segment_residual_estimates_match_reference(case, prob):
    """Every estimate the reference offers (residual_type 0/1/2, with and
    without scale_by_time, and residual2), on the state of each stage dump."""
    cs = pkg()
    g = golden("stage_" + case)
    ref = golden("segres_" + case)
    P = oracle_problem(prob)
    m, N = int(g["m"]), int(g["N"])
    seg = cs.tables.segment_tables(m)
    args = (P, m, N, g["t"], g["y"], g["y_dot"], g["z_tilde"], g["p"], float(g["alpha"]), float(g["tol"]), seg)
    for rt, sc in MODES:
        res, mx = O.segment_residual(*args, residual_type=rt, scale_by_time=sc)
        key = "t%d_s%d" % (rt, int(sc))
        np.testing.assert_allclose(res, ref["res_" + key], rtol=1e-10, atol=1e-12, err_msg=key)
        assert abs(mx - float(ref["max_" + key])) <= 1e-10 * abs(mx)
    res, mx = O.segment_residual(*args, residual2=True)
    np.testing.assert_allclose(res, ref["res2"], rtol=1e-10, atol=1e-12)
    assert abs(mx - float(ref["max2"])) <= 1e-10 * abs(mx)


def test_oracle_end_to_end_with_residual2_matches_reference():
    cs = pkg()
    g = golden("e2e_vdp_coarse_res2")
    P = oracle_problem("vdp_coarse")
    m = int(g["m"])
    r = O.solve(P, m, cs.tables.lobatto(m), cs.tables.segment_tables(m), residual2=True)
    assert r.success == bool(g["success"])
    assert r.N == g["t"].shape[0]
    assert r.jacobian_count == int(g["jacobian_counts"])
    assert r.residual_count == int(g["residual_counts"])
    assert r.nodes_after_remesh == list(g["nodes_after_remesh"])
    np.testing.assert_array_equal(np.round(np.array(r.norms), 8), g["norms"])
    np.testing.assert_array_equal(r.t, g["t"])
    np.testing.assert_allclose(r.y, g["y"], atol=1e-8, rtol=0)


@pytest.mark.parametrize("case,prob", STAGES[:3])
def test_oracle_chunked_newton_step_is_the_same(case, prob):
    """The memory-bounded Newton step (Jacobian, condensation and recovery
    over ranges of intervals, used for the large fixtures) gives the same
    numbers as the one-pass step, and both the reference's direction."""
    cs = pkg()
    g = golden("stage_" + case)
    P = oracle_problem(prob)
    m, N = int(g["m"]), int(g["N"])
    rk = cs.tables.lobatto(m)
    t, y, yd, zt, p, alpha = g["t"], g["y"], g["y_dot"], g["z_tilde"], g["p"], float(g["alpha"])
    f_q, y_tilde, f_a, f_b, r_bc = O.compute_f_q(P, m, N, rk, t, y, yd, zt, p, alpha)
    full = O.newton_step(P, m, N, rk, t, y, yd, zt, p, alpha, f_a, f_b, r_bc, y_tilde)
    for chunk in (1, 3, 7):
        part = O.newton_step(P, m, N, rk, t, y, yd, zt, p, alpha, f_a, f_b, r_bc, y_tilde, chunk=chunk)
        for a, b in zip(full, part):
            np.testing.assert_array_equal(a, b)
    np.testing.assert_allclose(full[0], g["delta_y"], rtol=0, atol=1e-10 * max(1.0, np.abs(g["delta_y"]).max()))
