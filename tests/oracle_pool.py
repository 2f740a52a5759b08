"""Oracle solves of many Van der Pol family instances in parallel, for the
batch parity tests: a pool of spawned, single-threaded worker processes
(spawned, so that no worker inherits the parent's CUDA state), each building
the family's numpy problem once.

solve_many(items) takes (m, theta, t, y, z, p) tuples -- an initial guess on
a mesh -- and returns, per item, a dict with the oracle's success, counts,
final mesh, solution and the nodes after each remesh."""
import os
from concurrent.futures import ProcessPoolExecutor
import multiprocessing as mp

_ENV = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
_W = {}


def _worker_init(root):
    import sys
    if root not in sys.path:
        sys.path.insert(0, root)


def _problem():
    if "P" not in _W:
        import importlib
        cs = importlib.import_module("collocation-solver-cuda_gb300")
        pr = cs.workloads.vdp_family_problem()

        class P:
            pass

        op = P()
        op.__dict__.update({k: v for k, v in pr.__dict__.items() if not k.startswith("_")})
        op.ny, op.nz, op.np = pr.size_y, pr.size_z, pr.size_p
        nf = cs.codegen.NumpyProblem(cs.codegen.ProblemCode(pr.sym))
        for k in ("f", "g", "Df", "Dg", "r", "Dr"):
            setattr(op, k, getattr(nf, k))
        _W["P"], _W["cs"] = op, cs
    return _W["P"], _W["cs"]


def _solve(item):
    import numpy as np
    from oracle import collocation_oracle as O
    m, theta, t, y, z, p = item
    P, cs = _problem()
    P.theta = np.asarray(theta, float)
    r = O.solve(P, m, cs.tables.lobatto(m), cs.tables.segment_tables(m), T0=t, Y0=y, Z0=z, P0=p)
    return dict(success=bool(r.success), N=int(r.N), newton_steps=int(r.jacobian_count),
                residual_evals=int(r.residual_count), remeshes=len(r.nodes_after_remesh), t=r.t, y=r.y, z=r.z,
                p=r.p)


def solve_many(items, procs=None):
    """Oracle solutions of every item, in order."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    procs = procs or min(len(items), os.cpu_count() or 1)
    old = {k: os.environ.get(k) for k in _ENV}
    for k in _ENV:
        os.environ[k] = "1"
    try:
        with ProcessPoolExecutor(max_workers=max(1, procs), mp_context=mp.get_context("spawn"),
                                 initializer=_worker_init, initargs=(root,)) as ex:
            # the longest (largest) meshes first, so that the pool's tail is short
            order = sorted(range(len(items)), key=lambda k: -len(items[k][2]))
            futs = {k: ex.submit(_solve, items[k]) for k in order}
            return [futs[k].result() for k in range(len(items))]
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
