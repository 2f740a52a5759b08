"""Front end (OCP parser + Pontryagin derivation + numpy codegen) against the
reference's generated problem modules (fixtures fe_*.npz made by running the
reference's OCP2ABVP.py; see tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, pkg

REF_NB = ["exContainerTransfer", "exFreespaceRocket", "exTrolley", "exUnderwaterVehicle"]
OCP_CASES = ["vdp", "vdp_coarse", "dint_param", "pend2", "vdp_ineq", "eqcon", "vdp_input", "vdp_svineq"]
# the reference's example OCP sources are read in place (never copied) from
# the checkout named by REF_DIR; these cases are skipped when it is not set
NB_TEXT_DIR = os.path.join(os.environ["REF_DIR"], "Notebook", "source") if os.environ.get("REF_DIR") else None


def _problem(case):
    cs = pkg()
    if case in OCP_CASES:
        return cs.ocp.Problem.from_file(os.path.join(GOLDEN, "ocp", case + ".ocp"))
    return cs.ocp.Problem.from_file(os.path.join(NB_TEXT_DIR, case))


@pytest.mark.parametrize("case", OCP_CASES + REF_NB)
def test_problem_functions_match_reference(case):
    cs = pkg()
    if case in REF_NB and (NB_TEXT_DIR is None or not os.path.exists(os.path.join(NB_TEXT_DIR, case))):
        pytest.skip("REF_DIR does not name a reference checkout with the example sources")
    g = golden("fe_" + case)
    pr = _problem(case)
    assert (pr.size_y, pr.size_z, pr.size_p) == (int(g["ny"]), int(g["nz"]), int(g["np"]))
    assert pr.size_inequality == int(g["n_ineq"]) and pr.size_sv_inequality == int(g["n_svineq"])
    nf = cs.codegen.NumpyProblem(cs.codegen.ProblemCode(pr.sym))
    th = pr.theta
    Y, Z, P, Y1, AL = g["Y"], g["Z"], g["P"], g["Y1"], g["ALPHA"]
    for k in range(Y.shape[0]):
        y, z, p = Y[k:k + 1], Z[k:k + 1], P[k]
        np.testing.assert_allclose(nf.f(y, z, p, th)[0], g["F"][k], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(nf.g(y, z, p, th, AL[k])[0], g["G"][k], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(nf.Df(y, z, p, th)[0], g["DF"][k], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(nf.Dg(y, z, p, th, AL[k])[0], g["DG"][k], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(nf.r(Y[k], Y1[k], p, th), g["R"][k], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(nf.Dr(Y[k], Y1[k], p, th), g["DR"][k], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("case", OCP_CASES)
def test_bvpdae_attributes_match_reference(case):
    g = golden("fe_" + case)
    pr = _problem(case)
    assert bool(g["has_bvpdae"])
    np.testing.assert_array_equal(pr.T0, g["T0"])
    np.testing.assert_array_equal(pr.Y0, g["Y0"])
    np.testing.assert_array_equal(pr.Z0, g["Z0"])
    np.testing.assert_array_equal(pr.P0, g["P0"])
    assert pr.tolerance == float(g["tolerance"])
    assert pr.maximum_nodes == int(g["maximum_nodes"])
    assert pr.maximum_newton_iterations == int(g["maximum_newton_iterations"])
    assert pr.maximum_mesh_refinements == int(g["maximum_mesh_refinements"])
    assert pr.output_file == str(g["output_file"])


def test_cuda_source_emits_all_functions():
    cs = pkg()
    pr = _problem("vdp")
    src = cs.codegen.cuda_problem_source(cs.codegen.ProblemCode(pr.sym))
    for fn in ("cs_f(", "cs_g(", "cs_Df(", "cs_Dg(", "cs_r(", "cs_Dr("):
        assert fn in src
    assert "pow(" not in src  # small integer powers are expanded


def test_parser_rejects_bad_statement():
    cs = pkg()
    with pytest.raises(cs.ocp.OcpSyntaxError):
        cs.ocp.parse_ocp("StateVariables = [x];\nFooBar = 3;\n")
    with pytest.raises(cs.ocp.OcpSyntaxError):
        cs.ocp.Problem("StateVariables = [x1, x2];\nDifferentialEquations = [x2];\n")


def test_theta_holds_constants():
    cs = pkg()
    pr = _problem("eqcon")
    assert pr.constant_names == ["a", "c"]
    np.testing.assert_array_equal(pr.theta, [2.0, 0.5])
