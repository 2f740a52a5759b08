"""Generate the stated-size fixtures of the two large single instances (the
pendulum chains of collocation-solver-cuda_gb300/workloads.py):

* K = 16: ny 64, nz 4, np 32; Nodes 8193, m = 5, tol 1e-6;
* K = 32: ny 128, nz 8, np 64; Nodes 16385, m = 4, tol 1e-8;

each solved by the oracle (oracle/collocation_oracle.py, the reference's
algorithm restated in numpy: partial-pivot LU condensation, the 8-partition
Householder BABD solve, line search, segment residual, remesh) from the
workload's own initial guess.  The oracle's Newton step runs over chunks of
256 intervals (the same numbers as one pass; tests/test_oracle_golden.py).

Stored per case (large_pend<K>.npz): success, counts (Newton, residual,
segment), the nodes after each remesh, the infinity-norm sequence, the final
N and mesh t, the maximum segment residual, the first Newton direction (dy on
every 16th node and the last, dp) and the solution (y, z on every 16th node
and the last; p).

Usage:  python tests/golden/make_large_golden.py [16] [32]
CPU only; minutes for K = 16, about an hour for K = 32 (BLAS on all cores).
"""
import importlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

STRIDE = 16
CHUNK = 256


def sub(a):
    """Rows 0, STRIDE, 2 STRIDE, ... and the last row."""
    idx = np.unique(np.r_[np.arange(0, a.shape[0], STRIDE), a.shape[0] - 1])
    return np.ascontiguousarray(a[idx])


def oracle_problem(cs, pr):
    class P:
        pass

    op = P()
    op.__dict__.update({k: v for k, v in pr.__dict__.items() if not k.startswith("_")})
    op.ny, op.nz, op.np = pr.size_y, pr.size_z, pr.size_p
    nf = cs.codegen.NumpyProblem(cs.codegen.ProblemCode(pr.sym))
    for k in ("f", "g", "Df", "Dg", "r", "Dr"):
        setattr(op, k, getattr(nf, k))
    return op


def make(K):
    from oracle import collocation_oracle as O
    cs = importlib.import_module("collocation-solver-cuda_gb300")
    c = cs.workloads.PENDULUM_CHAINS[K]
    m = c["m"]
    pr = cs.workloads.pendulum_chain_problem(K)
    P = oracle_problem(cs, pr)
    first = {}

    def trace(event, dy=None, dp=None):
        if event == "direction" and "dy" not in first:
            first["dy"], first["dp"] = dy.copy(), dp.copy()
        print("  [K=%d %.0f s] %s" % (K, time.time() - t0, event), flush=True)

    t0 = time.time()
    res = O.solve(P, m, cs.tables.lobatto(m), cs.tables.segment_tables(m), chunk=CHUNK, trace=trace, verbose=True)
    out = os.path.join(HERE, "large_pend%d.npz" % K)
    np.savez_compressed(
        out, K=K, m=m, nodes=c["nodes"], tol=c["tol"], stride=STRIDE, success=res.success, N=res.N,
        jacobian_counts=res.jacobian_count, residual_counts=res.residual_count, segment_counts=res.segment_count,
        nodes_after_remesh=np.array(res.nodes_after_remesh, dtype=np.int64), norms=np.array(res.norms),
        max_residual=res.max_residual, alpha=res.alpha, t=res.t, y=sub(res.y), z=sub(res.z), p=res.p,
        dy0=sub(first["dy"]), dp0=first["dp"], seconds=time.time() - t0)
    print("K=%d: %s, N %d, %d Newton, %d residuals, %.0f s -> %s" % (
        K, "solved" if res.success else "FAILED", res.N, res.jacobian_count, res.residual_count, time.time() - t0, out))


if __name__ == "__main__":
    for k in (sys.argv[1:] or ["16", "32"]):
        make(int(k))
