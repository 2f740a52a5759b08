"""The reference's four notebook example problems (container transfer,
free-space rocket, trolley, underwater vehicle: control- and
state-constrained OCPs that run the alpha continuation), solved on the GPU
from the guess the reference falls back to without their missing InputFile
data, against the oracle's solve from the same guess
(tests/golden/make_notebook_golden.py): same outcome, Newton and residual
counts, remeshes and final mesh (bit for bit), y, z, p within 1e-8 of their
scale.  The problems travel as this package's generated CUDA source
(GeneratedProblem), so the test needs neither sympy nor the reference."""
import numpy as np
import pytest

from conftest import golden, pkg

pytestmark = pytest.mark.gpu

NAMES = ["exContainerTransfer", "exFreespaceRocket", "exTrolley", "exUnderwaterVehicle"]


@pytest.mark.parametrize("name", NAMES)
def test_notebook_problem_matches_oracle(name):
    cs = pkg()
    g = golden("nb_" + name)
    gp = cs.GeneratedProblem.from_arrays(g)
    cp = cs.CompiledProblem(gp, int(g["m"]))
    bt = cs.Batch(cp, 1)
    bt.set_guess([(g["T0"], g["Y0"], g["Z0"])], g["P0"].reshape(1, -1))
    bt.solve(cs.default_opts(gp))
    s = bt.solution()[0]
    print("%s: GPU %s N %d Newton %d residuals %d remeshes %d; oracle %s N %d Newton %d" % (
        name, s["success"], s["N"], s["newton_steps"], s["residual_evals"], s["remeshes"], bool(g["success"]),
        int(g["N"]), int(g["jacobian_counts"])))
    assert s["success"] == bool(g["success"])
    assert (s["newton_steps"], s["residual_evals"], s["N"], s["remeshes"]) == \
           (int(g["jacobian_counts"]), int(g["residual_counts"]), int(g["N"]), len(g["nodes_after_remesh"]))
    np.testing.assert_array_equal(s["t"], g["t"])
    for k in ("y", "z", "p"):
        ref = g[k]
        np.testing.assert_allclose(s[k], ref, rtol=0, atol=1e-8 * max(1.0, np.abs(ref).max(initial=0.0)), err_msg=k)
