import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pkg():
    return importlib.import_module("collocation-solver-cuda_gb300")


class OracleProblem:
    """Problem object in the oracle's duck-typed interface, built from the
    package front end (parser + derivation + numpy codegen)."""

    def __init__(self, pr):
        cs = pkg()
        self.pr = pr
        self.__dict__.update({k: v for k, v in pr.__dict__.items() if not k.startswith("_")})
        self.ny, self.nz, self.np = pr.size_y, pr.size_z, pr.size_p
        pc = cs.codegen.ProblemCode(pr.sym)
        nf = cs.codegen.NumpyProblem(pc)
        for k in ("f", "g", "Df", "Dg", "r", "Dr"):
            setattr(self, k, getattr(nf, k))


def load_problem(name):
    cs = pkg()
    return cs.ocp.Problem.from_file(os.path.join(GOLDEN, "ocp", name + ".ocp"))


def oracle_problem(name):
    return OracleProblem(load_problem(name))


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
