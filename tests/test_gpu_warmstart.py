"""The learned warm start: trained on solutions of the batched solver, it
must lower the Newton work on held-out instances, and with the fallback every
instance the plain method solves is solved, to the same tolerance."""
import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def test_warm_start_gains_over_plain_guess():
    cs = pkg()
    ws = cs.warmstart
    fam = ws.vdp_family()
    solver = ws.BatchSolver(fam)
    train = cs.workloads.vdp_batch(1536, seed=1000, n_range=(32, 160))
    held = cs.workloads.vdp_batch(256, seed=7, n_range=(32, 160))
    X, Y, _ = ws.training_set(fam, solver, train)
    assert len(X) > 1200
    net = ws.Mlp(X.shape[1], Y.shape[1], width=256, depth=4, seed=0)
    net.fit_normalization(X, Y)
    net.train(X, Y, epochs=300, batch=256, lr=1e-3, seed=0)
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
