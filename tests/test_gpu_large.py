"""Large stage systems: the kernels with a global-memory slab per CTA
(blocked LU condensation, CTA-per-merge tree, CTA top solve), through the
C ABI.

* On the golden stage cases, the large-system layout gives the condensed
  blocks of the shared-memory layout to 1e-14 relative: the blocked LU
  performs the unblocked elimination's operations in the same order, and
  only the problem functions, compiled into other kernels, may round a
  product-sum differently (most cases agree bit for bit).  The Newton
  directions agree to 1e-12 (the Householder updates of the tree sum in
  another order).
* End-to-end with the large-system layout: the reference's golden solves
  (same Newton, residual and remesh counts, solutions within 1e-8).
* Pendulum chains of K = 16 (ny 64, nz 4, np 32, m 5: s = 340) and K = 32
  (ny 128, nz 8, np 64, m 4: s = 544), which only the large-system layout
  can hold, against the oracle: stage residual 1e-12, condensed blocks 1e-9,
  Newton directions 1e-8 (relative to the largest entry), segment residual
  1e-11, and whole solves (same counts, solutions within 1e-8).
"""
import numpy as np
import pytest

from conftest import OracleProblem, golden, load_problem, pkg
from oracle import collocation_oracle as O

pytestmark = pytest.mark.gpu

STAGES = [("vdp_n21_m4", "vdp"), ("vdp_n33_m5", "vdp"), ("dint_n33_m3", "dint_param"),
          ("pend2_n21_m5", "pend2"), ("econ_n17_m3", "eqcon")]
E2E = [("vdp_cfg1", "vdp"), ("pend2", "pend2"), ("vdp_ineq", "vdp_ineq"), ("vdp_svineq", "vdp_svineq")]


@pytest.fixture(scope="module")
def cs():
    c = pkg()
    c._lib.load()
    return c


_CP = {}


def compiled(cs, key, make_problem, m, layout):
    k = (key, m, layout)
    if k not in _CP:
        _CP[k] = cs.CompiledProblem(make_problem(), m, layout=layout)
    return _CP[k]


def _direction(cs, cp, t, y, yd, zt, p, alpha, theta=None):
    bt = cs.Batch(cp, 1)
    bt.set_state([(t, y, yd, zt)], np.asarray(p, float).reshape(1, -1),
                 None if theta is None else np.asarray(theta, float).reshape(1, -1))
    return bt, bt.stage_newton_direction(alpha)


@pytest.mark.parametrize("case,prob", STAGES)
def test_large_layout_matches_shared_memory_layout(cs, case, prob):
    g = golden("stage_" + case)
    m, N = int(g["m"]), int(g["N"])
    outs = []
    for layout in (1, 2):
        cp = compiled(cs, prob, lambda: load_problem(prob), m, layout)
        _, out = _direction(cs, cp, g["t"], g["y"], g["y_dot"], g["z_tilde"], g["p"], float(g["alpha"]))
        outs.append(out)
    small, big = outs
    rs, rb = small["rows"][:N - 1], big["rows"][:N - 1]
    np.testing.assert_allclose(rb, rs, rtol=1e-14, atol=1e-14 * max(1.0, np.abs(rs).max()))
    for k in ("dy", "dydot", "dzt", "dp"):
        a, b = np.asarray(big[k]), np.asarray(small[k])
        if a.size == 0:
            continue
        scale = max(1.0, np.abs(b).max())
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * scale, err_msg=k)


@pytest.mark.parametrize("case,prob", E2E)
def test_large_layout_end_to_end_matches_reference(cs, case, prob):
    g = golden("e2e_" + case)
    m = int(g["m"])
    pr = load_problem(prob)
    sol = cs.solver.solve_single(pr, m, layout=2)
    assert sol["success"] == bool(g["success"])
    assert sol["N"] == g["t"].shape[0]
    assert sol["newton_steps"] == int(g["jacobian_counts"])
    assert sol["residual_evals"] == int(g["residual_counts"])
    np.testing.assert_array_equal(sol["t"], g["t"])
    for k in ("y", "z", "p"):  # 1e-8 of each array's scale
        np.testing.assert_allclose(sol[k], g[k], atol=1e-8 * max(1.0, np.abs(g[k]).max(initial=0.0)), rtol=0)


# ------------------------------------------------------- pendulum chains ---
PEND = {16: 5, 32: 4}   # K -> m (the sizes of the large single-instance workloads)


def _pendulum(cs, K, nodes):
    theta0 = np.random.default_rng(0).uniform(-0.5, 0.5, K)
    return cs.ocp.Problem(cs.workloads.pendulum_ocp(K, theta0, nodes=nodes), name="pend%d" % K)


def _pend_state(cs, K, m, nodes, seed=3):
    """A generic state: the problem's initial input plus noise."""
    pr = _pendulum(cs, K, nodes)
    P = OracleProblem(pr)
    rk = cs.tables.lobatto(m)
    y, yd, zt = O.form_initial_input(P, m, nodes, np.asarray(pr.Y0, float), np.asarray(pr.Z0, float),
                                     np.asarray(pr.P0, float), rk)
    rng = np.random.default_rng(seed)
    y = y + 0.05 * rng.standard_normal(y.shape)
    yd = yd + 0.05 * rng.standard_normal(yd.shape)
    zt = zt + 0.05 * rng.standard_normal(zt.shape)
    p = np.asarray(pr.P0, float) + 0.05 * rng.standard_normal(pr.size_p)
    return pr, P, rk, np.asarray(pr.T0, float), y, yd, zt, p


@pytest.mark.parametrize("K", [16, 32])
def test_pendulum_stages_match_oracle(cs, K):
    m = PEND[K]
    nodes = 9
    pr, P, rk, t, y, yd, zt, p = _pend_state(cs, K, m, nodes)
    cp = compiled(cs, "pend%d" % K, lambda: pr, m, 0)
    alpha = 0.1
    # residual pieces
    bt = cs.Batch(cp, 1)
    bt.set_state([(t, y, yd, zt)], p.reshape(1, -1))
    norms, fa, fb = bt.stage_residual(alpha, pieces=True)
    f_q, y_tilde, f_a, f_b, r_bc = O.compute_f_q(P, m, nodes, rk, t, y, yd, zt, p, alpha)
    sc = max(1.0, np.abs(f_q).max())
    np.testing.assert_allclose(fa[:nodes - 1], f_a, rtol=0, atol=1e-12 * sc)
    np.testing.assert_allclose(fb[:nodes - 1], f_b, rtol=0, atol=1e-12 * sc)
    assert abs(norms[0] - np.abs(f_q).max()) <= 1e-12 * sc
    # condensed blocks and the Newton direction
    out = bt.stage_newton_direction(alpha)
    ny, npe = cp.ny, cp.np_eff
    J, V, D, W, B_0, B_n, V_n = O.construct_jacobian(P, m, nodes, rk, t, y, y_tilde, zt, p, alpha)
    A, C, H, b = O.reduce_jacobian(ny, cp.nz, cp.np, m, nodes, W, D, J, V, f_a, f_b)
    rows = out["rows"][:nodes - 1].reshape(nodes - 1, 2 * ny + npe + 1, ny)
    gA = np.transpose(rows[:, :ny, :], (0, 2, 1))
    gb = rows[:, 2 * ny + npe, :]
    np.testing.assert_allclose(gA, A.reshape(nodes - 1, ny, ny), rtol=0, atol=1e-9 * max(1.0, np.abs(A).max()))
    np.testing.assert_allclose(gb, b, rtol=0, atol=1e-9 * max(1.0, np.abs(b).max()))
    dy, dyd, dzt, dp = O.newton_step(P, m, nodes, rk, t, y, yd, zt, p, alpha, f_a, f_b, r_bc, y_tilde)
    scale = max(1.0, np.abs(dy).max())
    np.testing.assert_allclose(out["dy"][:nodes], dy, rtol=0, atol=1e-8 * scale)
    np.testing.assert_allclose(out["dp"][0], dp, rtol=0, atol=1e-8 * scale)
    np.testing.assert_allclose(out["dydot"][:nodes - 1].reshape(-1, ny), dyd, rtol=0,
                               atol=1e-8 * max(1.0, np.abs(dyd).max()))
    np.testing.assert_allclose(out["dzt"][:nodes - 1].reshape(-1, cp.nz), dzt, rtol=0,
                               atol=1e-8 * max(1.0, np.abs(dzt).max()))
    # segment residual
    res, mx = bt.stage_segment_residual(alpha, pr.tolerance)
    ref, ref_max = O.segment_residual(P, m, nodes, t, y, yd, zt, p, alpha, pr.tolerance, cs.tables.segment_tables(m))
    np.testing.assert_allclose(res[:nodes], ref, rtol=1e-11, atol=1e-12)
    assert abs(mx[0] - ref_max) <= 1e-11 * abs(ref_max)


@pytest.mark.parametrize("K", [16, 32])
def test_pendulum_solve_matches_oracle(cs, K):
    """Whole solves from a coarse 9-node guess: remeshes, the continuation
    and the Newton counts as the oracle's."""
    m = PEND[K]
    pr = _pendulum(cs, K, 9)
    cp = compiled(cs, "pend%d" % K, lambda: pr, m, 0)
    bt = cs.Batch(cp, 1)
    bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                 np.asarray(pr.P0, float).reshape(1, -1))
    bt.solve(cs.default_opts(pr))
    s = bt.solution()[0]
    P = OracleProblem(pr)
    ref = O.solve(P, m, cs.tables.lobatto(m), cs.tables.segment_tables(m))
    assert s["success"] == ref.success
    assert (s["N"], s["newton_steps"], s["residual_evals"]) == (ref.N, ref.jacobian_count, ref.residual_count)
    assert s["remeshes"] == len(ref.nodes_after_remesh)
    np.testing.assert_allclose(s["y"], ref.y, rtol=0, atol=1e-8)
    np.testing.assert_allclose(s["z"], ref.z, rtol=0, atol=1e-8)
    np.testing.assert_allclose(s["p"], ref.p, rtol=0, atol=1e-8)


# ------------------------------------------------------ reduced precision ---
@pytest.mark.parametrize("prec,tol", [("tf32", 1e-3), ("bf16", 1e-2)])
def test_reduced_precision_direction_close_to_fp64(cs, prec, tol):
    """The TF32 / BF16 tensor-core condensation is an inexact Jacobian: its
    blocks and Newton direction stay within `tol` (relative to the largest
    entry) of the FP64 ones (measured: TF32 2e-5 / 4e-5, BF16 2e-4 / 5e-4)."""
    pr = _pendulum(cs, 16, 65)
    outs = {}
    for p in ("fp64", prec):
        cp = cs.CompiledProblem(pr, 5, precision=p)
        bt = cs.Batch(cp, 1)
        bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                     np.asarray(pr.P0, float).reshape(1, -1))
        outs[p] = bt.stage_newton_direction(0.1)
    r0, r1 = outs["fp64"]["rows"][:64], outs[prec]["rows"][:64]
    assert np.abs(r1 - r0).max() <= tol * np.abs(r0).max()
    d0, d1 = outs["fp64"]["dy"][:65], outs[prec]["dy"][:65]
    assert np.abs(d1 - d0).max() <= tol * np.abs(d0).max()


@pytest.mark.parametrize("prec", ["tf32", "bf16"])
def test_reduced_precision_solve_reaches_fp64_oracle_solution(cs, prec):
    """Inexact Newton with an FP64 residual, line search and mesh error: the
    solve meets the FP64 tolerance on the oracle's mesh, and its states,
    costates and controls are within 1e-6 max-abs of the FP64 oracle's
    (measured: TF32 3e-10, BF16 7e-8)."""
    pr = _pendulum(cs, 16, 9)
    cp = cs.CompiledProblem(pr, 5, precision=prec)
    bt = cs.Batch(cp, 1)
    bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                 np.asarray(pr.P0, float).reshape(1, -1))
    bt.solve(cs.default_opts(pr))
    s = bt.solution()[0]
    ref = O.solve(OracleProblem(pr), 5, cs.tables.lobatto(5), cs.tables.segment_tables(5))
    assert s["success"] and ref.success
    assert s["N"] == ref.N
    assert s["last_norm"] < pr.tolerance and s["max_residual"] <= 1.0
    for k, rk in (("y", ref.y), ("z", ref.z), ("p", ref.p)):
        assert np.abs(s[k] - rk).max() < 1e-6, (k, np.abs(s[k] - rk).max())


@pytest.mark.parametrize("refine", [0, 2])
def test_tensor_core_tree_option_converges_on_small_chain(cs, refine):
    """The opt-in TF32 tree merges (precision "tf32-tree"): without
    refinement a more inexact direction (measured ~1e-2 relative), so more
    Newton steps, but the FP64 residual still drives the solve to the
    tolerance; with the default two FP64 refinement sweeps, the Newton count
    of the TF32 condensation with the FP64 tree (the refinement removes the
    tree's error; the condensation's own remains, which on this coarse mesh
    costs one step against FP64).  K = 16 from a coarse 9-node guess, within
    1e-5 of the FP64 oracle (measured 5e-7 unrefined)."""
    pr = _pendulum(cs, 16, 9)
    cp = cs.CompiledProblem(pr, 5, precision="tf32-tree")
    bt = cs.Batch(cp, 1)
    bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                 np.asarray(pr.P0, float).reshape(1, -1))
    bt.solve(cs.default_opts(pr, refine=refine))
    s = bt.solution()[0]
    ref = O.solve(OracleProblem(pr), 5, cs.tables.lobatto(5), cs.tables.segment_tables(5))
    assert s["success"] and s["N"] == ref.N
    assert np.abs(s["y"] - ref.y).max() < 1e-5
    if refine:
        cp1 = cs.CompiledProblem(pr, 5, precision="tf32")
        b1 = cs.Batch(cp1, 1)
        b1.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                     np.asarray(pr.P0, float).reshape(1, -1))
        b1.solve(cs.default_opts(pr))
        assert s["newton_steps"] == b1.solution()[0]["newton_steps"]


def test_pendulum8_hybrid_layout_matches_oracle(cs):
    """K = 8 (s1 = 102): blocked-LU condensation with the warp-per-merge
    tree, the automatic layout for this size; a whole solve from a coarse
    guess against the oracle."""
    th = np.random.default_rng(4).uniform(-0.5, 0.5, 8)
    pr = cs.ocp.Problem(cs.workloads.pendulum_ocp(8, th, nodes=9), name="pend8")
    cp = cs.CompiledProblem(pr, 4)
    bt = cs.Batch(cp, 1)
    bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                 np.asarray(pr.P0, float).reshape(1, -1))
    bt.solve(cs.default_opts(pr))
    s = bt.solution()[0]
    ref = O.solve(OracleProblem(pr), 4, cs.tables.lobatto(4), cs.tables.segment_tables(4))
    assert s["success"] == ref.success
    assert (s["N"], s["newton_steps"], s["residual_evals"]) == (ref.N, ref.jacobian_count, ref.residual_count)
    np.testing.assert_allclose(s["y"], ref.y, rtol=0, atol=1e-8)
    np.testing.assert_allclose(s["z"], ref.z, rtol=0, atol=1e-8)


# ------------------------------------------ the stated sizes, against the oracle ---
def _stated_size(cs, K, precision="fp64"):
    pr = cs.workloads.pendulum_chain_problem(K)
    cp = cs.CompiledProblem(pr, cs.workloads.PENDULUM_CHAINS[K]["m"], precision=precision)
    bt = cs.Batch(cp, 1)
    bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                 np.asarray(pr.P0, float).reshape(1, -1))
    return pr, cp, bt


def _rows(a, g):
    """The fixture's node rows: every `stride`-th node and the last."""
    n = a.shape[0]
    return a[np.unique(np.r_[np.arange(0, n, int(g["stride"])), n - 1])]


@pytest.mark.parametrize("K", [16, 32])
def test_pendulum_chain_at_stated_size_matches_oracle(cs, K):
    """Configs 2 and 4 at their stated sizes in FP64 (K = 16: Nodes 8193,
    m = 5, tol 1e-6; K = 32: Nodes 16385, m = 4, tol 1e-8) against the
    oracle's solve of the same instance from the same guess
    (tests/golden/make_large_golden.py): the first Newton direction within
    1e-8 of its scale, then the whole solve with the same Newton and residual
    counts, remeshes and final mesh, y, z, p within 1e-8 of their scale."""
    g = golden("large_pend%d" % K)
    pr, cp, bt = _stated_size(cs, K)
    N0 = len(pr.T0)
    d = bt.stage_newton_direction(0.1)
    sc = max(1.0, np.abs(g["dy0"]).max())
    np.testing.assert_allclose(_rows(d["dy"][:N0], g), g["dy0"], rtol=0, atol=1e-8 * sc)
    np.testing.assert_allclose(d["dp"][0], g["dp0"], rtol=0, atol=1e-8 * sc)
    del bt
    _, _, bt = _stated_size(cs, K)
    bt.solve(cs.default_opts(pr))
    s = bt.solution()[0]
    assert s["success"] == bool(g["success"])
    assert (s["newton_steps"], s["residual_evals"], s["N"], s["remeshes"]) == \
           (int(g["jacobian_counts"]), int(g["residual_counts"]), int(g["N"]), len(g["nodes_after_remesh"]))
    np.testing.assert_array_equal(s["t"], g["t"])
    for k in ("y", "z"):
        ref = g[k]
        np.testing.assert_allclose(_rows(s[k], g), ref, rtol=0, atol=1e-8 * max(1.0, np.abs(ref).max()), err_msg=k)
    np.testing.assert_allclose(s["p"], g["p"], rtol=0, atol=1e-8 * max(1.0, np.abs(g["p"]).max()))


# the stated error bound of the reduced-precision (tensor-core) condensation
# against the FP64 oracle, max-abs over y, z and p on the fixture's nodes
REDUCED_BOUND = 1e-8


@pytest.mark.parametrize("K,prec", [(16, "tf32"), (16, "bf16"), (32, "tf32"), (32, "bf16")])
def test_pendulum_chain_reduced_precision_error_against_oracle(cs, K, prec):
    """Configs 2 and 4 at their stated sizes with the TF32 / BF16 tensor-core
    condensation (inexact Newton with the FP64 residual, line search and mesh
    error): the solve reaches the tolerance on the oracle's final mesh and
    its states, costates, controls and parameters are within REDUCED_BOUND
    (max-abs) of the FP64 oracle's."""
    g = golden("large_pend%d" % K)
    pr, cp, bt = _stated_size(cs, K, prec)
    bt.solve(cs.default_opts(pr))
    s = bt.solution()[0]
    assert s["success"] and bool(g["success"])
    assert s["N"] == int(g["N"])
    np.testing.assert_array_equal(s["t"], g["t"])
    assert s["last_norm"] < float(g["tol"]) and s["max_residual"] <= 1.0
    err = max(np.abs(_rows(s["y"], g) - g["y"]).max(), np.abs(_rows(s["z"], g) - g["z"]).max(),
              np.abs(s["p"] - g["p"]).max())
    print("K=%d %s: max-abs error against the FP64 oracle %.3g (Newton %d, oracle %d)"
          % (K, prec, err, s["newton_steps"], int(g["jacobian_counts"])))
    assert err < REDUCED_BOUND


@pytest.mark.parametrize("prec", ["tf32", "bf16"])
def test_refinement_removes_the_tree_error(cs, prec):
    """FP64 iterative refinement of the direction (four sweeps) with the
    tree merges on the tensor cores: the low-precision tree adds an error
    far larger than the condensation's (measured at K = 16, 65 nodes: TF32
    5.8e-3 against 3.2e-5, BF16 5.5e-2 against 4.8e-4, relative to the FP64
    direction); after the sweeps only the condensation's error is left."""
    pr = _pendulum(cs, 16, 65)
    dy = {}
    for p, rf in (("fp64", 0), (prec, 0), (prec + "-tree", 0), (prec + "-tree", 4)):
        cp = cs.CompiledProblem(pr, 5, precision=p)
        bt = cs.Batch(cp, 1)
        bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                     np.asarray(pr.P0, float).reshape(1, -1))
        bt.set_opts(cs.default_opts(pr, refine=rf))
        dy[(p, rf)] = bt.stage_newton_direction(0.1)["dy"][:65]
    ref = dy[("fp64", 0)]
    err = {k: np.abs(v - ref).max() / np.abs(ref).max() for k, v in dy.items()}
    e_cond, e_tree, e_ref = err[(prec, 0)], err[(prec + "-tree", 0)], err[(prec + "-tree", 4)]
    print("%s: condensation %.3g, with the tree %.3g, after 4 refinement sweeps %.3g" % (prec, e_cond, e_tree, e_ref))
    assert e_tree > 10 * e_cond
    assert e_ref <= 1.5 * e_cond


def test_tensor_core_tree_with_refinement_keeps_the_fp64_newton_count(cs):
    """The TF32 tree merges at the stated size of config 2 (K = 16, 8193
    nodes) with FP64 iterative refinement of every direction: the solve takes
    the FP64 oracle's Newton and residual counts and lands within
    REDUCED_BOUND of its solution.  On this mesh a sweep contracts the tree's
    error by only ~0.4 (measured: 0.56 unrefined, 0.24, 0.094, 8.9e-3 after
    4, 9.7e-6 after 8 sweeps, relative to the FP64 direction), so this uses
    8 sweeps; the default 2 can cost a Newton step here.  (The BF16 tree is
    not refinable at this size: its error grows past 1 over the tree's
    levels, 4e6 relative, and a sweep amplifies it.)"""
    K = 16
    prec = "tf32-tree"
    g = golden("large_pend%d" % K)
    pr, cp, bt = _stated_size(cs, K, prec)
    assert cs.default_opts(pr).refine == 2
    bt.solve(cs.default_opts(pr, refine=8))
    s = bt.solution()[0]
    assert s["success"]
    assert (s["newton_steps"], s["residual_evals"], s["N"]) == \
           (int(g["jacobian_counts"]), int(g["residual_counts"]), int(g["N"]))
    err = max(np.abs(_rows(s["y"], g) - g["y"]).max(), np.abs(_rows(s["z"], g) - g["z"]).max(),
              np.abs(s["p"] - g["p"]).max())
    print("K=%d %s, 8 refinement sweeps: max-abs error against the FP64 oracle %.3g" % (K, prec, err))
    assert err < REDUCED_BOUND
