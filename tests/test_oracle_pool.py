"""The oracle process pool of the batch parity tests returns, per item, what
a direct oracle solve of that item returns."""
import numpy as np

from conftest import OracleProblem, pkg
from oracle import collocation_oracle as O


def test_pool_matches_direct_oracle_solves():
    from oracle_pool import solve_many
    cs = pkg()
    insts = cs.workloads.vdp_batch(3, seed=5, n_range=(12, 30))
    got = solve_many([(i.m, i.theta) + tuple(i.guess()) for i in insts], procs=2)
    P = OracleProblem(cs.workloads.vdp_family_problem())
    for inst, g in zip(insts, got):
        P.theta = inst.theta
        t, y, z, p = inst.guess()
        r = O.solve(P, inst.m, cs.tables.lobatto(inst.m), cs.tables.segment_tables(inst.m), T0=t, Y0=y, Z0=z, P0=p)
        assert (g["success"], g["N"], g["newton_steps"], g["residual_evals"]) == \
               (r.success, r.N, r.jacobian_count, r.residual_count)
        np.testing.assert_array_equal(g["y"], r.y)
        np.testing.assert_array_equal(g["p"], r.p)
