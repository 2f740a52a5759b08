"""Generate the fixtures of the reference's four notebook example problems
(Notebook/source/exContainerTransfer, exFreespaceRocket, exTrolley,
exUnderwaterVehicle), solved from the guess the reference itself falls back
to when an OCP's InputFile is missing (the examples name warm-start files
that the reference does not ship): the problem's own Nodes/FinalTime mesh,
state/control estimates or zeros, parameter estimates or ones.

The OCP sources are read in place from the reference checkout named by
REF_DIR and parsed by this package's front end; nothing of them is copied.
Each fixture (nb_<name>.npz) holds what a GPU test needs without the
reference: this package's generated CUDA problem functions and sizes, the
problem's solver settings and constants, the guess, and the oracle's solve
(oracle/collocation_oracle.py) from that guess with m = 4 (the reference
CLI's default): outcome, counts, remeshes, final mesh and solution.

Usage:  REF_DIR=<reference checkout> python tests/golden/make_notebook_golden.py [name ...]
CPU only; one process per problem; minutes each.
"""
import importlib
import os
import sys
import time
from multiprocessing import get_context

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
NAMES = ["exContainerTransfer", "exFreespaceRocket", "exTrolley", "exUnderwaterVehicle"]
M = 4


def make(name):
    sys.path.insert(0, ROOT)
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from oracle import collocation_oracle as O
    cs = importlib.import_module("collocation-solver-cuda_gb300")
    src = os.path.join(os.environ["REF_DIR"], "Notebook", "source", name)
    pr = cs.ocp.Problem.from_file(src)
    pc = cs.codegen.ProblemCode(pr.sym)

    class P:
        pass

    op = P()
    op.__dict__.update({k: v for k, v in pr.__dict__.items() if not k.startswith("_")})
    op.ny, op.nz, op.np = pr.size_y, pr.size_z, pr.size_p
    nf = cs.codegen.NumpyProblem(pc)
    for k in ("f", "g", "Df", "Dg", "r", "Dr"):
        setattr(op, k, getattr(nf, k))
    T0, Y0, Z0, P0 = (np.asarray(a, float) for a in (pr.T0, pr.Y0, pr.Z0, pr.P0))
    t0 = time.time()
    r = O.solve(op, M, cs.tables.lobatto(M), cs.tables.segment_tables(M), T0=T0, Y0=Y0, Z0=Z0, P0=P0)
    out = os.path.join(HERE, "nb_%s.npz" % name)
    np.savez_compressed(
        out, name=name, m=M, cuda_source=cs.codegen.cuda_problem_source(pc), ny=pc.ny, nz=pc.nz, np=pc.np,
        np_eff=pc.np_eff, nth=pc.nth, theta=np.asarray(pr.theta, float), tolerance=pr.tolerance,
        maximum_newton_iterations=pr.maximum_newton_iterations, maximum_mesh_refinements=pr.maximum_mesh_refinements,
        maximum_nodes=pr.maximum_nodes, size_inequality=pr.size_inequality, size_sv_inequality=pr.size_sv_inequality,
        T0=T0, Y0=Y0, Z0=Z0, P0=P0, success=r.success, N=r.N, jacobian_counts=r.jacobian_count,
        residual_counts=r.residual_count, nodes_after_remesh=np.array(r.nodes_after_remesh, dtype=np.int64),
        alpha=r.alpha, max_residual=r.max_residual, t=r.t, y=r.y, z=r.z, p=r.p, seconds=time.time() - t0)
    return "%s: %s, N %d, %d Newton, %d residuals, %d remeshes, alpha %.3g, %.0f s" % (
        name, "solved" if r.success else "FAILED", r.N, r.jacobian_count, r.residual_count,
        len(r.nodes_after_remesh), r.alpha, time.time() - t0)


if __name__ == "__main__":
    if not os.environ.get("REF_DIR"):
        sys.exit("set REF_DIR to the reference checkout (read-only), e.g. REF_DIR=/root/reference")
    names = sys.argv[1:] or NAMES
    with get_context("spawn").Pool(len(names)) as pool:
        for line in pool.imap_unordered(make, names):
            print(line, flush=True)
