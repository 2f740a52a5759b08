"""The learned warm start: trained on solutions of the batched solver, it
must lower the Newton work on held-out instances, and with the fallback every
instance the plain method solves is solved, to the same tolerance."""
import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vdp_net():
    """A network trained on 1,536 solutions of the batched solver (Van der Pol
    family, meshes of 32..160 intervals), shared by the tests below."""
    cs = pkg()
    ws = cs.warmstart
    fam = ws.vdp_family()
    solver = ws.BatchSolver(fam)
    train = cs.workloads.vdp_batch(1536, seed=1000, n_range=(32, 160))
    X, Y, _ = ws.training_set(fam, solver, train)
    net = ws.Mlp(X.shape[1], Y.shape[1], width=256, depth=4, seed=0)
    net.fit_normalization(X, Y)
    net.train(X, Y, epochs=300, batch=256, lr=1e-3, seed=0)
    return fam, solver, net, len(X)


def test_warm_start_gains_over_plain_guess(vdp_net):
    cs = pkg()
    ws = cs.warmstart
    fam, solver, net, n_train = vdp_net
    held = cs.workloads.vdp_batch(256, seed=7, n_range=(32, 160))
    assert n_train > 1200
    plain = solver.solve(held)
    final, fb, warm = ws.solve_warm(fam, solver, net, held)
    plain_ok = [s["success"] for s in plain]
    final_ok = [s["success"] for s in final]
    # the fallback keeps every instance the plain method solves
    assert all(f or not p for p, f in zip(plain_ok, final_ok))
    newton_plain = np.mean([s["newton_steps"] for s in plain])
    newton_warm = np.mean([s["newton_steps"] for s in warm])
    assert newton_warm < 0.7 * newton_plain, (newton_warm, newton_plain)
    assert len(fb) <= 0.1 * len(held)
    for s in final:
        if s["success"]:
            assert s["last_norm"] < 1e-6 and s["max_residual"] <= 1.0


def _family(cs, name):
    ws = cs.warmstart
    return ws.vdp_family() if name == "vdp" else ws.pendulum_family(8)


def _instances(cs, name, n, seed, n_range):
    if name == "vdp":
        return cs.workloads.vdp_batch(n, seed=seed, n_range=n_range, m_choices=(4,))
    return cs.workloads.pendulum_batch(n, K=8, seed=seed, n_range=n_range)


@pytest.mark.parametrize("name", ["vdp", "pendulum8"])
def test_device_warm_fill_matches_host_interpolation(name):
    """The device fill (trajectory vectors -> y, z at the mesh nodes, p,
    then the stage values) equals the host interpolation followed by the
    oracle's initial input, for both families."""
    from conftest import OracleProblem
    from oracle import collocation_oracle as O
    cs = pkg()
    ws = cs.warmstart
    fam = _family(cs, name)
    insts = _instances(cs, name, 5, 3, (20, 60))
    m = 4
    cp = cs.CompiledProblem(fam.problem, m)
    bt = cs.Batch(cp, len(insts))
    N, t, y, z, p, th = ws.pack_family(fam, insts)
    bt.set_guess_packed(N, t, y, z, p, th)
    V = np.random.default_rng(1).standard_normal((len(insts), fam.n_out)).astype(np.float32)
    d = cs.module.DeviceArray(V.shape, np.float32)
    d.upload(V)
    bt.warm_start(d.ptr, ws.N_NODES, fam.n_out)
    st = bt.state()
    P = OracleProblem(fam.problem)
    rk = cs.tables.lobatto(m)
    off = 0
    for b, inst in enumerate(insts):
        n = int(N[b])
        tb = t[off:off + n]
        yh, zh, ph = ws.guess_from_vector(V[b].astype(np.float64), tb, fam.final_time(inst), fam.ny, fam.nz, fam.np)
        np.testing.assert_allclose(st["y"][off:off + n], yh, rtol=0, atol=1e-12 * max(1.0, np.abs(yh).max()))
        np.testing.assert_allclose(st["z"][off:off + n], zh, rtol=0, atol=1e-12 * max(1.0, np.abs(zh).max()))
        np.testing.assert_array_equal(st["p"][b], ph)
        P.theta = fam.theta(inst)
        _, yd, zt = O.form_initial_input(P, m, n, st["y"][off:off + n], st["z"][off:off + n], st["p"][b], rk)
        np.testing.assert_allclose(st["ydot"][off:off + n - 1].reshape(-1, fam.ny), yd, rtol=1e-12,
                                   atol=1e-12 * max(1.0, np.abs(yd).max()))
        off += n


def test_pendulum_family_warm_start_gains_over_plain_guess():
    """The second warm-start family (pendulum chain K = 8, theta(0), T and the
    coupling as parameters): fewer Newton steps than the plain guess, no
    instance lost."""
    cs = pkg()
    ws = cs.warmstart
    fam = ws.pendulum_family(8)
    solver = ws.BatchSolver(fam)
    train = cs.workloads.pendulum_batch(1024, K=8, seed=1000, n_range=(32, 64))
    held = cs.workloads.pendulum_batch(128, K=8, seed=7, n_range=(32, 64))
    X, Y, _ = ws.training_set(fam, solver, train)
    assert len(X) > 900
    net = ws.Mlp(X.shape[1], Y.shape[1], width=256, depth=4, seed=0)
    net.fit_normalization(X, Y)
    net.train(X, Y, epochs=200, batch=256, lr=1e-3, seed=0)
    plain = solver.solve(held)
    final, fb, warm = ws.solve_warm(fam, solver, net, held)
    assert all(f["success"] or not p["success"] for p, f in zip(plain, final))
    newton_plain = np.mean([s["newton_steps"] for s in plain])
    newton_warm = np.mean([s["newton_steps"] for s in warm])
    assert newton_warm < newton_plain, (newton_warm, newton_plain)
    for s in final:
        if s["success"]:
            assert s["last_norm"] < 1e-6 and s["max_residual"] <= 1.0


def test_guess_and_solution_files_round_trip(tmp_path):
    """An MLP guess written as a solution file is read back by the OCP front
    end as InputFile; a batch's solutions written per instance read back
    exactly (the reference's reader format)."""
    cs = pkg()
    ws = cs.warmstart
    fam = ws.vdp_family()
    inst = cs.workloads.vdp_batch(1, seed=3, n_range=(40, 40), m_choices=(4,))[0]
    net = ws.Mlp(4, fam.n_out, width=64, depth=3, seed=0)
    path = str(tmp_path / "guess.data")
    assert ws.write_guess_file(fam, net, inst, path) == 0
    err, t, y, z, p = cs.io.bvpdae_read_data(path)
    assert err == 0 and t.shape == (41,) and y.shape == (41, fam.ny) and z.shape == (41, fam.nz)
    text = open(cs.workloads.VDP_FAMILY_OCP).read().replace("OutputFile", 'InputFile = "%s";\nOutputFile' % path)
    pr = cs.ocp.Problem(text, name="vdp_from_guess")
    np.testing.assert_array_equal(pr.T0, t)
    # per-instance solution files of a solved batch
    solver = ws.BatchSolver(fam)
    insts = cs.workloads.vdp_batch(3, seed=4, n_range=(32, 48), m_choices=(4,))
    N, tt, yy, zz, pp, th = ws.pack_family(fam, insts)
    bt = cs.Batch(solver.cp(4), 3)
    bt.set_guess_packed(N, tt, yy, zz, pp, th)
    bt.solve(solver.opts)
    st = ws.write_solution_files(bt, str(tmp_path / "sol_%d.data"))
    assert st == [0, 0, 0]
    for b, s in enumerate(bt.solution()):
        err, t2, y2, z2, p2 = cs.io.bvpdae_read_data(str(tmp_path / ("sol_%d.data" % b)))
        assert err == 0
        np.testing.assert_array_equal(t2, s["t"])
        np.testing.assert_array_equal(y2, s["y"])


def test_speculative_fallback_gives_the_sequential_results():
    """Starting the plain-guess solves early (for every instance still
    iterating, at the first check or once 3 % of a group is), on a second
    thread or as spares inside the warm batch, changes no instance's result
    against falling back after the warm solve."""
    cs = pkg()
    ws = cs.warmstart
    fam = ws.vdp_family()
    insts = cs.workloads.vdp_batch(96, seed=23, n_range=(32, 128))
    # an untrained network with a wide output scale: poor guesses, so that a
    # good part of the batch fails warm and falls back
    net = ws.Mlp(4, fam.n_out, width=64, depth=3, seed=2)
    X = np.array([fam.features(i) for i in insts], np.float32)
    rng = np.random.default_rng(0)
    net.fit_normalization(X, (1.5 * rng.standard_normal((len(insts), fam.n_out))).astype(np.float32))
    solver = ws.BatchSolver(fam)
    runner = ws.WarmRunner(fam, solver, net, insts)
    base = runner.run(warm=True, speculate=0)
    assert base[1] > 0
    def same(got):
        assert got[:2] == base[:2]
        for a, b in zip(got[2], base[2]):
            assert (a["success"], a.get("fallback", False), a["newton_steps"], a["residual_evals"], a["N"]) == \
                   (b["success"], b.get("fallback", False), b["newton_steps"], b["residual_evals"], b["N"])
            np.testing.assert_array_equal(a["y"], b["y"])
            np.testing.assert_array_equal(a["t"], b["t"])

    for frac in (1.0, 0.03):
        got = runner.run(warm=True, speculate=frac)
        if frac == 1.0:
            assert sum(n for _, n, _ in runner.times["speculated"]) >= base[1]
        same(got)
    # the plain copies inside the warm batch (spares): started at the first
    # check, once 3 % of a group is in Newton, or once none is
    paired = ws.WarmRunner(fam, solver, net, insts, spares=True)
    for at in (1.0, 0.03, 0.0):
        got = paired.run(warm=True, spare_at=at)
        started = sum(n for _, n, _ in paired.times["speculated"])
        assert started >= base[1]
        same(got)
    # without the warm start the spares stay parked: the plain batched solve
    plain = runner.run(warm=False)
    got = paired.run(warm=False)
    assert got[:2] == plain[:2] and sum(n for _, n, _ in paired.times["speculated"]) == 0
    for a, b in zip(got[2], plain[2]):
        assert (a["newton_steps"], a["N"]) == (b["newton_steps"], b["N"])
        np.testing.assert_array_equal(a["y"], b["y"])


def _held_out_sample(cs, per_m, seed):
    """`per_m` random instances of each m from the benchmark's held-out batch
    (8192 Van der Pol instances, seed 7, N ~ U{32..2048} intervals)."""
    held = cs.workloads.vdp_batch(8192, seed=7)
    rng = np.random.default_rng(seed)
    pick = []
    for m in (3, 4, 5):
        idx = [k for k, inst in enumerate(held) if inst.m == m]
        pick += sorted(int(k) for k in rng.choice(idx, per_m, replace=False))
    return [held[k] for k in pick]


def _split(st, k0, N):
    """Instance rows of a packed state: (t, y, z) of the node slots."""
    o = int(np.sum(N[:k0]))
    n = int(N[k0])
    return st["t"][o:o + n].copy(), st["y"][o:o + n].copy(), st["z"][o:o + n].copy()


def _assert_same_solve(s, ref, label):
    assert s["success"] == ref["success"], label
    assert (s["newton_steps"], s["residual_evals"], s["N"], s["remeshes"]) == \
           (ref["newton_steps"], ref["residual_evals"], ref["N"], ref["remeshes"]), label
    np.testing.assert_array_equal(s["t"], ref["t"], err_msg=label)
    for k in ("y", "z", "p"):
        sc = max(1.0, np.abs(ref[k]).max(initial=0.0))
        np.testing.assert_allclose(s[k], ref[k], rtol=0, atol=1e-8 * sc, err_msg="%s %s" % (label, k))


def test_warm_started_bench_instances_match_oracle_from_the_same_guess(vdp_net):
    """48 instances of the benchmark's own held-out batch (16 per m, meshes up
    to 2048 intervals), warm-started as the benchmark does (device MLP,
    device fill), against the oracle solving each from the same device-filled
    guess: same outcome, Newton and residual counts, remeshes and final mesh
    (bit for bit), y, z, p within 1e-8 of their scale.  Separately, where the
    warm-started solve ends on the mesh of the oracle's solve from the plain
    guess, the two solutions agree within the accuracy the tolerance gives
    (both residuals below 1e-6): 1e-6 of the scale."""
    from oracle_pool import solve_many
    cs = pkg()
    ws = cs.warmstart
    fam, solver, net, _ = vdp_net
    insts = _held_out_sample(cs, 16, seed=0)
    runner = ws.WarmRunner(fam, solver, net, insts)
    net.predict_device(runner.dX, len(runner.instances), runner.dY)
    items, sols = [], []
    for g in runner.groups:
        bt = g["bt"]
        bt.reset()
        bt.warm_start(runner.dY.ptr + 4 * g["first"] * net.n_out, ws.N_NODES, net.n_out)
        st = bt.state()
        for b in range(g["n"]):
            inst = runner.instances[g["first"] + b]
            t, y, z = _split(st, b, st["N"])
            items.append((inst.m, inst.theta, t, y, z, st["p"][b].copy()))
        bt.solve(solver.opts)
        sols += bt.solution()
    plain_items = [(i.m, i.theta) + tuple(i.guess()) for i in runner.instances]
    refs = solve_many(items + plain_items)
    warm_ref, plain_ref = refs[:len(items)], refs[len(items):]
    assert sum(s["success"] for s in sols) >= 40
    assert max(s["N"] for s in sols) > 1500
    same_mesh, worst = 0, 0.0
    for k, (s, ref, pref) in enumerate(zip(sols, warm_ref, plain_ref)):
        _assert_same_solve(s, ref, "instance %d (m %d)" % (k, runner.instances[k].m))
        if s["success"] and pref["success"] and s["N"] == pref["N"] and np.array_equal(s["t"], pref["t"]):
            same_mesh += 1
            for key in ("y", "z", "p"):
                sc = max(1.0, np.abs(pref[key]).max(initial=0.0))
                d = np.abs(s[key] - pref[key]).max(initial=0.0) / sc
                worst = max(worst, d)
    print("warm vs plain-guess oracle: %d of %d on the same final mesh, max difference %.3g of scale"
          % (same_mesh, len(sols), worst))
    assert worst <= 1e-6


def test_spares_parked_filled_and_started_at_the_end():
    """The spare half of a paired batch (cs_batch_set_spares) is parked by the
    guess, keeps its guess through the warm start, stays parked in a solve
    with trigger < 0, and, with a trigger of 0 in a later solve, runs exactly
    for the failed primaries (a short iteration limit makes failures): each
    such spare equals the plain solve of its instance, bit for bit; the
    spares of succeeded primaries stay parked."""
    cs = pkg()
    ws = cs.warmstart
    fam = ws.vdp_family()
    insts = [i for i in cs.workloads.vdp_batch(64, seed=29, n_range=(32, 96)) if i.m == 4]
    n = len(insts)
    opts = cs.default_opts(fam.problem, max_nodes=20000, max_iter=6)
    solver = ws.BatchSolver(fam, opts)
    net = ws.Mlp(4, fam.n_out, width=64, depth=3, seed=3)
    X = np.array([fam.features(i) for i in insts], np.float32)
    rng = np.random.default_rng(1)
    net.fit_normalization(X, (1.5 * rng.standard_normal((n, fam.n_out))).astype(np.float32))
    N, t, y, z, p, th = ws.pack_family(fam, insts + insts)
    bt = cs.Batch(solver.cp(4), 2 * n)
    with pytest.raises(cs._lib.CsError):
        bt.set_spares(n + 1, 0)
    bt.set_spares(n, -1)
    bt.set_guess_packed(N, t, y, z, p, th)
    st = bt.statuses()
    assert (st[:n] == 0).all() and (st[n:] == 6).all()
    dX = cs.module.DeviceArray(X.shape, np.float32)
    dX.upload(X)
    dY = cs.module.DeviceArray((n, net.n_out), np.float32)
    net.predict_device(dX, n, dY)
    bt.warm_start(dY, ws.N_NODES, net.n_out)
    s0 = bt.state()
    o = int(N[:n].sum())
    np.testing.assert_array_equal(s0["y"][o:], y[o:])
    assert not np.array_equal(s0["y"][:o], y[:o])
    bt.solve(opts)
    st = bt.statuses()
    assert (st[n:] == 6).all() and set(st[:n].tolist()) <= {3, 4}
    failed = [int(k) for k in np.flatnonzero(st[:n] == 4)]
    done = [int(k) for k in np.flatnonzero(st[:n] == 3)]
    assert failed
    bt.set_spares(n, 0)
    bt.solve(opts)
    st = bt.statuses()
    assert set(st[[n + k for k in failed]].tolist()) <= {3, 4}
    assert (st[[n + k for k in done]] == 6).all()
    sols = bt.solution([n + k for k in failed])
    ref = solver.solve([insts[k] for k in failed])
    for a, b in zip(sols, ref):
        assert (a["status"], a["newton_steps"], a["residual_evals"], a["N"]) == \
               (b["status"], b["newton_steps"], b["residual_evals"], b["N"])
        np.testing.assert_array_equal(a["t"], b["t"])
        np.testing.assert_array_equal(a["y"], b["y"])
