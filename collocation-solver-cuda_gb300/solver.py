"""Host-side mirror of the reference solver's Python interface, running on the
GB300 kernels through the C ABI.

`collocation_solver_parallel(m, problem)` keeps the behaviour of the
reference driver (collocation_solver_parallel_2d_shared.py:36-251): the same
printed summary, the benchmark-counts file under ./benchmark_performance/,
the appended test_results_m_*.txt line and the solution file written with
bvpdae_write_data when the continuation finished.  The stage functions keep
the reference's names and argument meaning for one instance.
"""
import os
import pathlib
import time

import numpy as np

from .io import bvpdae_write_data
from .module import Batch, CompiledProblem, default_opts

_COMPILED = {}


def compiled(problem, m):
    key = (id(problem), m)
    cp = _COMPILED.get(key)
    if cp is None or cp.problem is not problem:
        cp = CompiledProblem(problem, m)
        _COMPILED[key] = cp
    return cp


def solve_single(problem, m=4, T0=None, Y0=None, Z0=None, P0=None, theta=None, opts=None, layout=0):
    """Solve one instance from its initial guess (defaults: the problem's
    BvpDae T0/Y0/Z0/P0).  Returns the solution dict of Batch.solution().
    layout: kernel layout of CompiledProblem (0 automatic)."""
    cp = compiled(problem, m) if layout == 0 else CompiledProblem(problem, m, layout=layout)
    bt = Batch(cp, 1)
    t = np.asarray(problem.T0 if T0 is None else T0, dtype=np.float64)
    y = np.asarray(problem.Y0 if Y0 is None else Y0, dtype=np.float64)
    z = np.asarray(problem.Z0 if Z0 is None else Z0, dtype=np.float64)
    p = np.asarray(problem.P0 if P0 is None else P0, dtype=np.float64).reshape(1, -1)
    th = None if theta is None else np.asarray(theta, dtype=np.float64).reshape(1, -1)
    bt.set_guess([(t, y, z)], p, th)
    bt.solve(opts if opts is not None else default_opts(problem))
    return bt.solution()[0]


def _write_benchmark(fname, counts, total_time):
    try:
        with open(fname, "w") as f:
            for label, key in (("Initial input", "initial"), ("Residual", "residual"), ("Jacobian", "jacobian"),
                               ("Reduce Jacobian", "jacobian"), ("Recover BABD", "jacobian"),
                               ("Segment Residual", "segment")):
                f.write("%s time: %s\n" % (label, counts.get(key + "_time", 0.0)))
                f.write("%s counts: %d\n" % (label, counts.get(key, 0)))
            f.write("Total time: {}\n".format(total_time))
    except OSError:
        print("Write time failed!")


def collocation_solver_parallel(m=4, problem=None, write_files=True):
    """Solve `problem` (an ocp.Problem) like the reference driver does."""
    print("m = {}".format(m))
    if problem is None:
        raise ValueError("problem is required")
    alpha_m = 1e-6 if (problem.size_inequality > 0 or problem.size_sv_inequality > 0) else 0.1
    t0 = time.time()
    sol = solve_single(problem, m)
    total = time.time() - t0
    print("Maximum residual: {}".format(sol["max_residual"]))
    print("Elapsed time: {}".format(total))
    example_name = problem.output_file.split(".")[0]
    M = 8
    if write_files:
        bdir = "./benchmark_performance/"
        pathlib.Path(bdir).mkdir(0o755, parents=True, exist_ok=True)
        counts = dict(initial=1 + sol["remeshes"], residual=sol["residual_evals"], jacobian=sol["newton_steps"],
                      segment=sol["segment_evals"])
        _write_benchmark(bdir + example_name + "_parallel_benchmark_M_{}.data".format(M), counts, total)
        if sol["alpha"] <= alpha_m:
            err = bvpdae_write_data(problem.output_file, sol["N"], problem.size_y, problem.size_z, problem.size_p,
                                    sol["t"], sol["y"], sol["z"], sol["p"])
            if err != 0:
                print("Write file failed.")
        with open("test_results_m_{}_residual2_{}_residualType_{}_scaleTime_{}_scaleInitial_{}.txt".format(
                m, False, 1, True, False), "a") as f:
            if sol["success"]:
                f.write("{} solved successfully. alpha = {}. Elapsed time: {}(s).\n".format(example_name, sol["alpha"], total))
            else:
                f.write("{} solved unsuccessfully. alpha = {}. Elapsed time: {}(s).\n".format(example_name, sol["alpha"], total))
    print("Problem solved successfully." if sol["success"] else "Problem solved unsuccessfully.")
    return sol


# ---------------------------------------------------------------- stages ---
def form_initial_input_parallel(problem, m, N, y0, z0, p0):
    """y' = f at the linearly interpolated stage points (CS:287-356); returns
    (y, y_dot, z_tilde) with the reference's shapes."""
    cp = compiled(problem, m)
    bt = Batch(cp, 1)
    bt.set_guess([(np.linspace(0.0, 1.0, N), np.asarray(y0, float), np.asarray(z0, float))],
                 np.asarray(p0, float).reshape(1, -1))
    st = bt.state()
    return np.asarray(y0, float), st["ydot"][:N - 1].reshape((N - 1) * m, cp.ny), \
        st["zt"][:N - 1].reshape((N - 1) * m, cp.nz)
