"""GB300-native collocation solver for the BVP-DAEs of nonlinear optimal
control problems (drop-in for the Newton inner loop of
UW-OCP/Collocation-Solver-CUDA).

Import with importlib (the directory name contains hyphens):

    import importlib
    cs = importlib.import_module("collocation-solver-cuda_gb300")
"""
from . import tables, ocp, codegen, io  # noqa: F401
