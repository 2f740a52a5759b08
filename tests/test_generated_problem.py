"""GeneratedProblem: a problem carried as its generated CUDA source and
settings (no sympy on the solving machine) has the front-end problem's
sizes, constants and solver settings, and round-trips through plain arrays."""
import numpy as np

from conftest import load_problem, pkg


def test_generated_problem_round_trip():
    cs = pkg()
    pr = load_problem("vdp_ineq")
    gp = cs.GeneratedProblem.from_problem(pr, name="vdp_ineq")
    pc = cs.codegen.ProblemCode(pr.sym)
    assert gp.cuda_source == cs.codegen.cuda_problem_source(pc)
    assert (gp.size_y, gp.size_z, gp.size_p, gp.code.np_eff, gp.code.nth) == (pc.ny, pc.nz, pc.np, pc.np_eff, pc.nth)
    arrays = dict(cuda_source=gp.cuda_source, ny=pc.ny, nz=pc.nz, np=pc.np, np_eff=pc.np_eff, nth=pc.nth,
                  theta=gp.theta, tolerance=pr.tolerance, maximum_newton_iterations=pr.maximum_newton_iterations,
                  maximum_mesh_refinements=pr.maximum_mesh_refinements, maximum_nodes=pr.maximum_nodes,
                  size_inequality=pr.size_inequality, size_sv_inequality=pr.size_sv_inequality, name="vdp_ineq")
    back = cs.GeneratedProblem.from_arrays({k: np.asarray(v) for k, v in arrays.items()})
    assert back.cuda_source == gp.cuda_source
    for k in ("size_y", "size_z", "size_p", "tolerance", "maximum_nodes", "size_inequality", "size_sv_inequality"):
        assert getattr(back, k) == getattr(pr, k), k
    np.testing.assert_array_equal(back.theta, np.asarray(pr.theta, float).reshape(-1))
