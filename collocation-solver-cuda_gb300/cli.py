"""Command-line entry, the drop-in for the reference's
`run_2d_shared.sh <ocp> [m]` (run_2d_shared.sh:1-5), which translates the OCP
with OCP2ABVP.py and runs collocation_solver_parallel_2d_shared.py -m m.

    python cli.py <ocp file> [-m M]

Parses and derives the OCP in process (no generated bvp_problem.py), solves it
on the GPU and writes, in the current directory, what the reference writes:
the solution file named by OutputFile, benchmark_performance/<name>_parallel_
benchmark_M_8.data and the test_results_m_*.txt line.
"""
import argparse
import importlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    ap = argparse.ArgumentParser(description="Solve an optimal control problem with the GB300 collocation solver.")
    ap.add_argument("ocp", help="plain-text OCP definition")
    ap.add_argument("-m", type=int, choices=[3, 4, 5, 6, 7, 8, 9, 10], default=4,
                    help="number of collocation points")
    args = ap.parse_args(argv)
    cs = importlib.import_module(os.path.basename(HERE))
    print("Solving %s" % args.ocp)
    print("Solve the optimal control problem with {} collocation points.".format(args.m))
    problem = cs.ocp.Problem.from_file(args.ocp)
    sol = cs.solver.collocation_solver_parallel(args.m, problem)
    return 0 if sol["success"] else 1


if __name__ == "__main__":
    sys.exit(main())
