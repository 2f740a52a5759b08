"""The command-line drop-in for the reference's run_2d_shared.sh <ocp> [m]."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden, pkg

PKG_DIR = os.path.join(ROOT, "collocation-solver-cuda_gb300")


def test_cli_rejects_an_m_the_reference_rejects():
    p = subprocess.run([sys.executable, os.path.join(PKG_DIR, "cli.py"), "x.ocp", "-m", "2"], capture_output=True,
                       text=True)
    assert p.returncode != 0 and "invalid choice" in p.stderr


@pytest.mark.gpu
def test_run_2d_shared_writes_what_the_reference_writes(tmp_path):
    """Config 1 (Van der Pol, 101 nodes, m = 4) through the script: the
    solution file (BVPDAEReadWriteData format) holds the reference's solution
    to 1e-8, and the benchmark and results files are written."""
    cs = pkg()
    shutil.copy(os.path.join(GOLDEN, "ocp", "vdp.ocp"), tmp_path)
    p = subprocess.run(["bash", os.path.join(PKG_DIR, "run_2d_shared.sh"), "vdp.ocp", "4"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    g = golden("e2e_vdp_cfg1")
    err, t, y, z, pp = cs.io.bvpdae_read_data(str(tmp_path / "vdp.data"))
    assert err == 0
    np.testing.assert_array_equal(np.asarray(t), g["t"])
    np.testing.assert_allclose(np.asarray(y), g["y"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(np.asarray(z), g["z"], rtol=0, atol=1e-8)
    # the same layout line by line as the reference's file
    ours = (tmp_path / "vdp.data").read_text().split("\n")
    ref = str(g["output_text"]).split("\n")
    assert len(ours) == len(ref)
    assert [len(a.split()) for a in ours] == [len(b.split()) for b in ref]
    assert os.path.exists(tmp_path / "benchmark_performance")
    assert any(f.startswith("test_results_m_") for f in os.listdir(tmp_path))
