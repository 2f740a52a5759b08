"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
golden fixtures of the reference.

Tolerances: stage residual pieces and segment residuals 1e-12 relative (same
formulas, different summation order); condensed blocks 1e-9 and Newton
directions 1e-8 (different but stable factorizations: LU of the stage system
is the same, the BABD system uses a tree of Householder merges instead of the
reference's 8 sequential partitions); end-to-end solutions 1e-8 max-abs with
identical Newton iteration counts, residual counts and final meshes.
"""
import numpy as np
import pytest

from conftest import golden, load_problem, oracle_problem, pkg
from oracle import collocation_oracle as O

pytestmark = pytest.mark.gpu

STAGES = [("vdp_n21_m4", "vdp"), ("vdp_n33_m5", "vdp"), ("dint_n33_m3", "dint_param"),
          ("pend2_n21_m5", "pend2"), ("econ_n17_m3", "eqcon")]
E2E = [("vdp_cfg1", "vdp"), ("vdp_coarse", "vdp_coarse"), ("dint_param", "dint_param"), ("vdp_input", "vdp_input"),
       ("pend2", "pend2"), ("vdp_ineq", "vdp_ineq"), ("vdp_svineq", "vdp_svineq"), ("vdp_m7", "vdp"),
       ("eqcon", "eqcon")]


@pytest.fixture(scope="module")
def cs():
    c = pkg()
    c._lib.load()
    return c


_CP = {}


def compiled(cs, name, m):
    key = (name, m)
    if key not in _CP:
        pr = load_problem(name)
        _CP[key] = cs.CompiledProblem(pr, m)
    return _CP[key]


def _batch_with_state(cs, cp, g):
    bt = cs.Batch(cp, 1)
    bt.set_state([(g["t"], g["y"], g["y_dot"], g["z_tilde"])], g["p"].reshape(1, -1))
    return bt


@pytest.mark.parametrize("case,prob", STAGES)
def test_stage_residual(cs, case, prob):
    g = golden("stage_" + case)
    m, N = int(g["m"]), int(g["N"])
    cp = compiled(cs, prob, m)
    bt = _batch_with_state(cs, cp, g)
    norms, fa, fb = bt.stage_residual(float(g["alpha"]), pieces=True)
    P = oracle_problem(prob)
    f_q, _, f_a, f_b, r_bc = O.compute_f_q(P, m, N, cs.tables.lobatto(m), g["t"], g["y"], g["y_dot"],
                                           g["z_tilde"], g["p"], float(g["alpha"]))
    np.testing.assert_allclose(fa[:N - 1], f_a, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(fb[:N - 1], f_b, rtol=1e-12, atol=1e-12)
    assert abs(norms[0] - np.abs(f_q).max()) <= 1e-12 * max(1.0, np.abs(f_q).max())
    # and the reference's own numbers
    np.testing.assert_allclose(fa[:N - 1], g["f_a"], rtol=1e-11, atol=1e-11)


@pytest.mark.parametrize("case,prob", STAGES)
def test_stage_newton_direction(cs, case, prob):
    g = golden("stage_" + case)
    m, N = int(g["m"]), int(g["N"])
    cp = compiled(cs, prob, m)
    bt = _batch_with_state(cs, cp, g)
    out = bt.stage_newton_direction(float(g["alpha"]))
    ny, npe = cp.ny, cp.np_eff
    rows = out["rows"][:N - 1].reshape(N - 1, 2 * ny + npe + 1, ny)  # column-major blocks
    A = np.transpose(rows[:, :ny, :], (0, 2, 1))
    C = np.transpose(rows[:, ny:2 * ny, :], (0, 2, 1))
    H = np.transpose(rows[:, 2 * ny:2 * ny + npe, :], (0, 2, 1))
    b = rows[:, 2 * ny + npe, :]
    gA = g["A"].reshape(N - 1, ny, ny)
    gH = g["H"].reshape(N - 1, ny, -1)
    np.testing.assert_allclose(A, gA, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(C, np.broadcast_to(np.eye(ny), C.shape), atol=0)
    np.testing.assert_allclose(H, gH[:, :, :npe], rtol=1e-9, atol=1e-9)
    assert np.all(gH[:, :, npe:] == 0)
    np.testing.assert_allclose(b, g["b"], rtol=1e-9, atol=1e-9)
    # full Newton direction against the reference's (partitioned QR + recovery)
    scale = max(1.0, np.abs(g["delta_y"]).max())
    np.testing.assert_allclose(out["dy"][:N], g["delta_y"], rtol=0, atol=1e-8 * scale)
    np.testing.assert_allclose(out["dp"][0], g["delta_p"], rtol=0, atol=1e-8 * scale)
    dyd = out["dydot"][:N - 1].reshape((N - 1) * m, ny)
    np.testing.assert_allclose(dyd, g["delta_y_dot"], rtol=0, atol=1e-8 * max(1.0, np.abs(g["delta_y_dot"]).max()))
    if cp.nz:
        dzt = out["dzt"][:N - 1].reshape((N - 1) * m, cp.nz)
        np.testing.assert_allclose(dzt, g["delta_z_tilde"], rtol=0,
                                   atol=1e-8 * max(1.0, np.abs(g["delta_z_tilde"]).max()))


@pytest.mark.parametrize("case,prob", STAGES)
def test_stage_segment_residual_and_remesh(cs, case, prob):
    g = golden("stage_" + case)
    m, N = int(g["m"]), int(g["N"])
    cp = compiled(cs, prob, m)
    bt = _batch_with_state(cs, cp, g)
    res, mx = bt.stage_segment_residual(float(g["alpha"]), float(g["tol"]))
    np.testing.assert_allclose(res[:N], g["seg_residual"], rtol=1e-11, atol=1e-12)
    assert abs(mx[0] - float(g["seg_max"])) <= 1e-11 * abs(float(g["seg_max"]))
    # remesh with the synthetic residual of the fixture: exact node arithmetic
    Nn = bt.stage_remesh(g["remesh_residual"])
    assert int(Nn[0]) == int(g["remesh_N"])
    st = bt.state()
    n = int(Nn[0])
    np.testing.assert_array_equal(st["t"][:n], g["remesh_t"])
    np.testing.assert_array_equal(st["y"][:n], g["remesh_y"])
    # stage values formed on the new mesh (y' = f at interpolated points)
    P = oracle_problem(prob)
    _, yd, zt = O.form_initial_input(P, m, n, g["remesh_y"], g["remesh_z"], g["p"], cs.tables.lobatto(m))
    np.testing.assert_allclose(st["ydot"][:n - 1].reshape(-1, cp.ny), yd, rtol=1e-12, atol=1e-12)
    if cp.nz:
        np.testing.assert_allclose(st["zt"][:n - 1].reshape(-1, cp.nz), zt, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("case,prob", E2E)
def test_end_to_end_matches_reference(cs, case, prob):
    g = golden("e2e_" + case)
    m = int(g["m"])
    pr = load_problem(prob)
    sol = cs.solver.solve_single(pr, m)
    assert sol["success"] == bool(g["success"])
    assert sol["N"] == g["t"].shape[0]
    assert sol["newton_steps"] == int(g["jacobian_counts"])
    assert sol["residual_evals"] == int(g["residual_counts"])
    assert sol["remeshes"] == len(g["nodes_after_remesh"])
    np.testing.assert_array_equal(sol["t"], g["t"])
    # 1e-8 of each array's scale (a state constraint's multiplier reaches ~300)
    for k in ("y", "z", "p"):
        np.testing.assert_allclose(sol[k], g[k], atol=1e-8 * max(1.0, np.abs(g[k]).max(initial=0.0)), rtol=0)
    assert abs(sol["max_residual"] - float(g["max_residual"])) <= 1e-6 * max(1.0, float(g["max_residual"]))


def test_batch_equals_independent_solves(cs):
    """Instances of one batch (different initial conditions through the
    constants, different meshes and final times) give the same results as the
    oracle run on each instance alone."""
    pr = load_problem("vdp_family")
    m = 4
    cp = compiled(cs, "vdp_family", m)
    rng = np.random.default_rng(5)
    B = 6
    meshes, thetas = [], []
    for b in range(B):
        N = int(rng.integers(20, 60))
        T = float(rng.uniform(2, 6))
        t = np.linspace(0.0, T, N)
        meshes.append((t, np.zeros((N, cp.ny)), np.zeros((N, cp.nz))))
        thetas.append([rng.uniform(-1.5, 1.5), rng.uniform(-1.5, 1.5), float(np.exp(rng.uniform(np.log(0.3), np.log(3))))])
    thetas = np.array(thetas)
    bt = cs.Batch(cp, B)
    bt.set_guess(meshes, np.ones((B, cp.np)), thetas)
    bt.solve(cs.default_opts(pr, max_nodes=20000))
    sols = bt.solution()
    P = oracle_problem("vdp_family")
    P.maximum_nodes = 20000
    for b in range(B):
        P.theta = thetas[b]
        ref = O.solve(P, m, cs.tables.lobatto(m), cs.tables.segment_tables(m), T0=meshes[b][0], Y0=meshes[b][1],
                      Z0=meshes[b][2], P0=np.ones(cp.np))
        s = sols[b]
        assert s["success"] == ref.success
        assert s["N"] == ref.N and s["newton_steps"] == ref.jacobian_count and s["residual_evals"] == ref.residual_count
        assert np.abs(s["y"] - ref.y).max() < 1e-8
        assert np.abs(s["z"] - ref.z).max() < 1e-8


def test_plain_batch_sample_matches_oracle(cs):
    """32 random instances of the batched plain-method workload (4096 Van der
    Pol instances, seed 1: x0, T, r per instance, N ~ U{32..2048} intervals,
    m in {3, 4, 5}), solved in one batch per m from the plain guess, against
    the oracle on each instance alone: same outcome, Newton and residual
    counts, remeshes and final mesh (bit for bit), y, z, p within 1e-8 of
    their scale."""
    from oracle_pool import solve_many
    insts = cs.workloads.vdp_batch(4096, seed=1)
    rng = np.random.default_rng(3)
    pick = [insts[int(k)] for k in sorted(rng.choice(len(insts), 32, replace=False))]
    assert {i.m for i in pick} == {3, 4, 5}
    solver = cs.warmstart.BatchSolver(cs.warmstart.vdp_family())
    sols = solver.solve(pick)
    refs = solve_many([(i.m, i.theta) + tuple(i.guess()) for i in pick])
    assert sum(r["success"] for r in refs) >= 28
    for k, (s, ref) in enumerate(zip(sols, refs)):
        label = "instance %d (m %d, %d intervals)" % (k, pick[k].m, pick[k].intervals)
        assert s["success"] == ref["success"], label
        assert (s["newton_steps"], s["residual_evals"], s["N"], s["remeshes"]) == \
               (ref["newton_steps"], ref["residual_evals"], ref["N"], ref["remeshes"]), label
        np.testing.assert_array_equal(s["t"], ref["t"], err_msg=label)
        for key in ("y", "z", "p"):
            sc = max(1.0, np.abs(ref[key]).max(initial=0.0))
            np.testing.assert_allclose(s[key], ref[key], rtol=0, atol=1e-8 * sc, err_msg=label + " " + key)


def test_failing_instances_match_oracle(cs):
    """Instances of the Van der Pol batch whose Newton iteration does not
    converge within the iteration limit: same failure, same counts (including
    the repeated rejected line searches) and same final iterate as the
    oracle."""
    from conftest import OracleProblem
    pr = cs.workloads.vdp_family_problem()
    insts = cs.workloads.vdp_batch(4096, seed=1)
    pick = [insts[i] for i in (209, 420, 629, 1125)]
    P = OracleProblem(pr)
    P.maximum_newton_iterations = 30
    for inst in pick:
        cp = compiled(cs, "vdp_family", inst.m)
        bt = cs.Batch(cp, 1)
        t, y, z, p = inst.guess()
        bt.set_guess([(t, y, z)], p.reshape(1, -1), inst.theta.reshape(1, -1))
        bt.solve(cs.default_opts(pr, max_iter=30))
        s = bt.solution()[0]
        P.theta = inst.theta
        ref = O.solve(P, inst.m, cs.tables.lobatto(inst.m), cs.tables.segment_tables(inst.m), T0=t, Y0=y, Z0=z, P0=p)
        assert s["success"] == ref.success
        assert (s["newton_steps"], s["residual_evals"], s["N"]) == (ref.jacobian_count, ref.residual_count, ref.N)
        assert np.abs(s["y"] - ref.y).max() < 1e-8


@pytest.mark.parametrize("case,prob", STAGES)
def test_stage_segment_residual_estimates(cs, case, prob):
    """The reference's other segment-residual estimates (residual_type 0 and
    2, without scale_by_time, residual2) against its own numbers."""
    g = golden("stage_" + case)
    ref = golden("segres_" + case)
    m = int(g["m"])
    cp = compiled(cs, prob, m)
    bt = _batch_with_state(cs, cp, g)
    pr = load_problem(prob)
    for rt in (0, 1, 2):
        for sc in (True, False):
            bt.set_opts(cs.default_opts(pr, residual_type=rt, scale_by_time=int(sc), residual2=0))
            res, mx = bt.stage_segment_residual(float(g["alpha"]), float(g["tol"]))
            key = "t%d_s%d" % (rt, int(sc))
            np.testing.assert_allclose(res[:int(g["N"])], ref["res_" + key], rtol=1e-11, atol=1e-12, err_msg=key)
            assert abs(mx[0] - float(ref["max_" + key])) <= 1e-11 * abs(float(ref["max_" + key]))
    bt.set_opts(cs.default_opts(pr, residual2=1))
    res, mx = bt.stage_segment_residual(float(g["alpha"]), float(g["tol"]))
    np.testing.assert_allclose(res[:int(g["N"])], ref["res2"], rtol=1e-11, atol=1e-12)
    assert abs(mx[0] - float(ref["max2"])) <= 1e-11 * abs(float(ref["max2"]))


def test_end_to_end_residual2_matches_reference(cs):
    g = golden("e2e_vdp_coarse_res2")
    m = int(g["m"])
    pr = load_problem("vdp_coarse")
    sol = cs.solver.solve_single(pr, m, opts=cs.default_opts(pr, residual2=1))
    assert sol["success"] == bool(g["success"])
    assert sol["N"] == g["t"].shape[0]
    assert sol["newton_steps"] == int(g["jacobian_counts"])
    assert sol["residual_evals"] == int(g["residual_counts"])
    assert sol["remeshes"] == len(g["nodes_after_remesh"])
    np.testing.assert_array_equal(sol["t"], g["t"])
    np.testing.assert_allclose(sol["y"], g["y"], atol=1e-8, rtol=0)
    np.testing.assert_allclose(sol["z"], g["z"], atol=1e-8, rtol=0)


def test_autotuned_condensation_gives_identical_solves(cs):
    """The shape tuner times its candidates on the batch and keeps the
    fastest; every candidate performs the same per-entry elimination, so the
    tuned solve is bit-identical to the untuned one."""
    pr = load_problem("vdp_family")
    cp = cs.CompiledProblem(pr, 4)
    insts = cs.workloads.vdp_batch(64, seed=21, n_range=(32, 400), m_choices=(4,))
    fam = cs.warmstart.vdp_family()
    N, t, y, z, p, th = cs.warmstart.pack_family(fam, insts)
    bt = cs.Batch(cp, len(insts))
    bt.set_guess_packed(N, t, y, z, p, th)
    opts = cs.default_opts(pr, max_nodes=20000)
    bt.solve(opts)
    before = bt.solution()
    bt.reset()
    r = bt.autotune(reps=2)
    assert r["candidates"] >= 2 and r["lanes"] in (4, 8, 16, 32) and r["ms"] <= r["default_ms"]
    bt.reset()
    bt.solve(opts)
    after = bt.solution()
    for s0, s1 in zip(before, after):
        assert (s0["newton_steps"], s0["residual_evals"], s0["N"]) == (s1["newton_steps"], s1["residual_evals"], s1["N"])
        np.testing.assert_array_equal(s0["y"], s1["y"])


@pytest.mark.parametrize("m", [2, 6, 8, 9, 10])
def test_extreme_collocation_orders_match_oracle(cs, m):
    """The orders not pinned by a reference solve (3, 4, 5 and 7 are; the
    reference's CLI allows 3..10, the tables go down to 2): a whole solve
    against the oracle, with the tables computed here (the reference's m = 10
    table has a known missing entry)."""
    pr = load_problem("vdp")
    cp = compiled(cs, "vdp", m)
    ref = O.solve(oracle_problem("vdp"), m, cs.tables.lobatto(m), cs.tables.segment_tables(m))
    sol = cs.solver.solve_single(pr, m)
    assert sol["success"] == ref.success
    assert (sol["N"], sol["newton_steps"], sol["residual_evals"]) == (ref.N, ref.jacobian_count, ref.residual_count)
    np.testing.assert_allclose(sol["y"], ref.y, rtol=0, atol=1e-8)


def _dense_direction(ny, npar, N, A, C, H, b, B_0, B_n, V_n, r_bc):
    """The condensed Newton system solved densely (the mathematical answer)."""
    n = N - 1
    sz = N * ny + npar
    M = np.zeros((sz, sz))
    rhs = np.zeros(sz)
    for i in range(n):
        rows = slice(i * ny, (i + 1) * ny)
        M[rows, i * ny:(i + 1) * ny] = A[rows]
        M[rows, (i + 1) * ny:(i + 2) * ny] = C[rows]
        M[rows, N * ny:] = H[rows]
        rhs[rows] = b[i]
    M[n * ny:, :ny], M[n * ny:, n * ny:N * ny], M[n * ny:, N * ny:] = B_0, B_n, V_n
    rhs[n * ny:] = -r_bc
    x = np.linalg.solve(M, rhs)
    return x[:N * ny].reshape(N, ny), x[N * ny:]


@pytest.mark.parametrize("N", [2, 5])
def test_short_meshes_solve_the_newton_system_exactly(cs, N):
    """Meshes with fewer than 9 nodes (one interval: no tree level at all).
    The reference's partitioned BABD solve (8 partitions of (N-1)//8 nodes,
    solve_babd_system.py:93-106) is wrong there -- its partition indices
    collapse to 0 -- and so is the oracle that restates it; the tree solve
    here is checked against a dense solve of the same condensed system."""
    m = 4
    cp = compiled(cs, "vdp", m)
    P = oracle_problem("vdp")
    rk = cs.tables.lobatto(m)
    t = np.linspace(0.0, 2.0, N)
    rng = np.random.default_rng(2)
    y0 = 0.3 * rng.standard_normal((N, cp.ny))
    z0 = 0.3 * rng.standard_normal((N, cp.nz))
    p = 0.5 + 0.3 * rng.random(cp.np)
    y, yd, zt = O.form_initial_input(P, m, N, y0, z0, p, rk)
    bt = cs.Batch(cp, 1)
    bt.set_state([(t, y, yd, zt)], p.reshape(1, -1))
    out = bt.stage_newton_direction(0.1)
    f_q, y_tilde, f_a, f_b, r_bc = O.compute_f_q(P, m, N, rk, t, y, yd, zt, p, 0.1)
    J, V, D, W, B_0, B_n, V_n = O.construct_jacobian(P, m, N, rk, t, y, y_tilde, zt, p, 0.1)
    A, C, H, b = O.reduce_jacobian(cp.ny, cp.nz, cp.np, m, N, W, D, J, V, f_a, f_b)
    dy, dp = _dense_direction(cp.ny, cp.np, N, A, C, H, b, B_0, B_n, V_n, r_bc)
    scale = max(1.0, np.abs(dy).max())
    np.testing.assert_allclose(out["dy"][:N], dy, rtol=0, atol=1e-10 * scale)
    np.testing.assert_allclose(out["dp"][0], dp, rtol=0, atol=1e-10 * scale)
    # the reference's partitioned solve misses it on these meshes
    dy_ref, _ = O.solve_babd(cp.ny, cp.np, N, A, C, H, b, B_0, B_n, V_n, r_bc)
    assert np.abs(dy_ref - dy).max() > 1e-3 * scale


def test_empty_batch_is_refused(cs):
    cp = compiled(cs, "vdp", 4)
    with pytest.raises(Exception):
        cs.Batch(cp, 0)


def test_nan_instance_fails_alone(cs):
    """An instance whose guess holds a NaN fails at the iteration limit
    without touching its batch-mates, which solve exactly as they do alone."""
    pr = cs.workloads.vdp_family_problem()
    insts = [i for i in cs.workloads.vdp_batch(64, seed=31) if i.m == 4][:4]
    cp = compiled(cs, "vdp_family", 4)
    opts = cs.default_opts(pr, max_nodes=20000)
    guesses = [inst.guess() for inst in insts]
    alone = []
    for inst, (t, y, z, p) in zip(insts, guesses):
        b1 = cs.Batch(cp, 1)
        b1.set_guess([(t, y, z)], p.reshape(1, -1), inst.theta.reshape(1, -1))
        b1.solve(opts)
        alone.append(b1.solution()[0])
    meshes = [(t, y.copy(), z) for t, y, z, _ in guesses]
    meshes[2][1][3, 1] = np.nan
    bt = cs.Batch(cp, len(insts))
    bt.set_guess(meshes, np.stack([g[3] for g in guesses]), np.stack([i.theta for i in insts]))
    bt.solve(opts)
    sols = bt.solution()
    # the NaN never leaves the instance: every trial norm is NaN, no step is
    # accepted, and it stops at the Newton iteration limit (numpy's dense solve
    # in the oracle raises or returns on a NaN matrix depending on the LAPACK
    # build, so the oracle is not asked here)
    assert not sols[2]["success"]
    assert sols[2]["fail_reason"] == 1 and sols[2]["newton_steps"] == opts.max_iter
    for k in (0, 1, 3):
        assert sols[k]["success"] == alone[k]["success"]
        assert (sols[k]["newton_steps"], sols[k]["N"]) == (alone[k]["newton_steps"], alone[k]["N"])
        np.testing.assert_array_equal(sols[k]["y"], alone[k]["y"])


def test_fused_upper_levels_give_the_per_level_bits(cs):
    """The upper tree levels, top system and their back substitution in one
    CTA per instance (automatic path) give bit for bit the solves of one
    launch per tree level (babd_path 2): counts, meshes, solutions."""
    pr = cs.workloads.vdp_family_problem()
    insts = [i for i in cs.workloads.vdp_batch(96, seed=41, n_range=(2, 700)) if i.m == 4][:24]
    cp = compiled(cs, "vdp_family", 4)
    guesses = [inst.guess() for inst in insts]
    meshes = [(t, y, z) for t, y, z, _ in guesses]
    P = np.stack([g[3] for g in guesses])
    TH = np.stack([i.theta for i in insts])
    out = []
    for path in (0, 2):
        bt = cs.Batch(cp, len(insts))
        bt.set_guess(meshes, P, TH)
        bt.solve(cs.default_opts(pr, max_nodes=20000, babd_path=path))
        out.append(bt.solution())
    assert sum(s["success"] for s in out[0]) >= len(insts) // 2
    for a, b in zip(*out):
        assert (a["success"], a["newton_steps"], a["residual_evals"], a["N"]) == \
               (b["success"], b["newton_steps"], b["residual_evals"], b["N"])
        np.testing.assert_array_equal(a["y"], b["y"])
        np.testing.assert_array_equal(a["z"], b["z"])


def test_fused_upper_levels_on_mixed_mesh_sizes(cs):
    """One batch with meshes of 2 to 700 nodes: instances whose whole tree is
    inside the fused levels (or has no level at all) next to ones with levels
    below them; same bits as one launch per level."""
    pr = load_problem("vdp_family")
    cp = compiled(cs, "vdp_family", 3)
    rng = np.random.default_rng(8)
    sizes = [2, 3, 5, 9, 17, 33, 65, 300, 700, 4]
    meshes, thetas = [], []
    for N in sizes:
        t = np.linspace(0.0, float(rng.uniform(2, 5)), N)
        meshes.append((t, np.zeros((N, cp.ny)), np.zeros((N, cp.nz))))
        thetas.append([rng.uniform(-1, 1), rng.uniform(-1, 1), float(np.exp(rng.uniform(np.log(0.5), np.log(2))))])
    out = []
    for path in (0, 2):
        bt = cs.Batch(cp, len(sizes))
        bt.set_guess(meshes, np.ones((len(sizes), cp.np)), np.array(thetas))
        bt.solve(cs.default_opts(pr, max_nodes=20000, babd_path=path))
        out.append(bt.solution())
    for a, b in zip(*out):
        assert (a["success"], a["newton_steps"], a["residual_evals"], a["N"]) == \
               (b["success"], b["newton_steps"], b["residual_evals"], b["N"])
        np.testing.assert_array_equal(a["y"], b["y"])
        np.testing.assert_array_equal(a["p"], b["p"])


def test_progress_hook_sees_every_check(cs):
    """cs_batch_set_progress: called after every check of the Newton phase
    with the instances still iterating; the statuses may be read from it; the
    solve's results do not change."""
    pr = load_problem("vdp_family")
    cp = compiled(cs, "vdp_family", 4)
    insts = [i for i in cs.workloads.vdp_batch(32, seed=3, n_range=(32, 200)) if i.m == 4][:6]
    guesses = [inst.guess() for inst in insts]
    meshes = [(t, y, z) for t, y, z, _ in guesses]
    P, TH = np.stack([g[3] for g in guesses]), np.stack([i.theta for i in insts])
    opts = cs.default_opts(pr, max_nodes=20000)
    seen = []
    bt = cs.Batch(cp, len(insts))
    bt.set_guess(meshes, P, TH)
    bt.set_progress(lambda active, steps: seen.append((active, steps, tuple(bt.statuses()))))
    bt.solve(opts)
    hooked = bt.solution()
    bt.set_progress(None)
    assert seen and all(0 <= a <= len(insts) for a, _, _ in seen)
    steps = [s for _, s, _ in seen]
    assert steps == sorted(steps) and steps[-1] > 0
    # the last check ends the last Newton phase: nobody is iterating any more
    # (converged ones may still await their segment residual)
    assert seen[-1][0] == 0 and all(st not in (0, 1) for st in seen[-1][2])
    bt2 = cs.Batch(cp, len(insts))
    bt2.set_guess(meshes, P, TH)
    bt2.solve(opts)
    for a, b in zip(hooked, bt2.solution()):
        assert (a["success"], a["newton_steps"], a["N"]) == (b["success"], b["newton_steps"], b["N"])
        np.testing.assert_array_equal(a["y"], b["y"])


def test_line_search_trial_count_changes_no_result(cs):
    """cs_opts.ls_grow only splits a line search's trials over super-steps
    (taken in the reference's order): a batch with failing and line-searching
    instances solves to the same bits and counts with 1, 2 and all 20 trials
    after a search that rejected some."""
    pr = load_problem("vdp_family")
    cp = cs.CompiledProblem(pr, 4)
    insts = cs.workloads.vdp_batch(64, seed=31, n_range=(32, 400), m_choices=(4,))
    fam = cs.warmstart.vdp_family()
    N, t, y, z, p, th = cs.warmstart.pack_family(fam, insts)
    bt = cs.Batch(cp, len(insts))
    bt.set_guess_packed(N, t, y, z, p, th)
    runs = []
    for grow in (0, 1, 2):
        bt.reset()
        bt.profile_reset(timing=False)
        bt.solve(cs.default_opts(pr, max_nodes=20000, ls_grow=grow))
        runs.append((bt.solution(), bt.profile()["super_steps"]))
    base, _ = runs[0]
    assert sum(s["residual_evals"] > 2 * s["newton_steps"] + 2 for s in base) > 0  # some searches rejected trials
    for sols, _ in runs[1:]:
        for a, b in zip(sols, base):
            assert (a["status"], a["newton_steps"], a["residual_evals"], a["N"]) == \
                   (b["status"], b["newton_steps"], b["residual_evals"], b["N"])
            np.testing.assert_array_equal(a["y"], b["y"])
