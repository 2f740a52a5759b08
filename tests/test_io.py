"""Solution-file format: byte-identical to the files the reference writes."""
import os

import numpy as np

from conftest import golden, pkg


def test_write_matches_reference_bytes(tmp_path):
    cs = pkg()
    g = golden("e2e_vdp_cfg1")
    fn = os.path.join(tmp_path, "out.data")
    t, y, z, p = g["t"], g["y"], g["z"], g["p"]
    assert cs.io.bvpdae_write_data(fn, t.shape[0], y.shape[1], z.shape[1], p.shape[0], t, y, z, p) == 0
    assert open(fn).read() == str(g["output_text"])


def test_read_write_round_trip(tmp_path):
    cs = pkg()
    rng = np.random.default_rng(0)
    N, ny, nz, npar = 7, 3, 2, 1
    t, y, z, p = np.linspace(0, 1, N), rng.standard_normal((N, ny)), rng.standard_normal((N, nz)), rng.standard_normal(npar)
    fn = os.path.join(tmp_path, "rt.data")
    assert cs.io.bvpdae_write_data(fn, N, ny, nz, npar, t, y, z, p) == 0
    err, t2, y2, z2, p2 = cs.io.bvpdae_read_data(fn)
    assert err == 0
    for a, b in ((t, t2), (y, y2), (z, z2), (p, p2)):
        np.testing.assert_array_equal(a, b)


def test_read_missing_file_reports_error(tmp_path):
    cs = pkg()
    err, t, y, z, p = cs.io.bvpdae_read_data(os.path.join(tmp_path, "nope.data"))
    assert err == 1 and t == [] and p == []
