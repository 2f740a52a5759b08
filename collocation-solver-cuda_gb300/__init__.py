"""GB300-native collocation solver for the BVP-DAEs of nonlinear optimal
control problems (drop-in for the Newton inner loop of
UW-OCP/Collocation-Solver-CUDA).

Import with importlib (the directory name contains hyphens):

    import importlib
    cs = importlib.import_module("collocation-solver-cuda_gb300")
    prob = cs.ocp.Problem.from_file("vdp.ocp")
    sol = cs.solver.solve_single(prob, m=4)

The GPU path needs libcs_gb300.so (built by build.py) and a CUDA device; there
is no CPU fallback.
"""
from . import tables, ocp, codegen, io, _lib, module, solver, build, workloads, warmstart  # noqa: F401
from .ocp import Problem  # noqa: F401
from .module import Batch, CompiledProblem, GeneratedProblem, default_opts  # noqa: F401
