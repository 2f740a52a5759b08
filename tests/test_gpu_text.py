"""Solution files formatted on the GPU (cs_format_solutions) against the host
writer (io.bvpdae_write_data, byte-identical to the reference's writer,
BVPDAEReadWriteData.py:337-364) on the same values: solved batches of two
families, and a batch whose values are arbitrary bit patterns (NaN, inf,
subnormals, signed zeros)."""
import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def _host_text(cs, bt):
    cp = bt.cp
    out = []
    for s in bt.solution():
        parts = ["nt:\n{}\nt:\n".format(s["N"])]
        parts.append("".join(cs.io._fmt(v) + " " for v in s["t"]))
        parts.append("\nny:\n{}\ny:\n".format(cp.ny))
        parts += ["".join(cs.io._fmt(v) + " " for v in row) + "\n" for row in s["y"]]
        parts.append("nz:\n{}\nz:\n".format(cp.nz))
        parts += ["".join(cs.io._fmt(v) + " " for v in row) + "\n" for row in s["z"]]
        parts.append("np:\n{}\np:\n".format(cp.np))
        parts.append("".join(cs.io._fmt(v) + " " for v in s["p"]))
        out.append("".join(parts).encode())
    return out


def _check(cs, bt):
    text, off = bt.solution_text()
    host = _host_text(cs, bt)
    assert len(off) == bt.B + 1 and off[0] == 0 and off[-1] == len(text)
    for b, h in enumerate(host):
        assert text[off[b]:off[b + 1]] == h, "instance %d" % b


@pytest.mark.parametrize("family", ["vdp", "pendulum8"])
def test_device_files_equal_host_writer_on_solved_batches(tmp_path, family):
    cs = pkg()
    ws = cs.warmstart
    if family == "vdp":
        fam = ws.vdp_family()
        insts = cs.workloads.vdp_batch(40, seed=8, n_range=(32, 400), m_choices=(4,))
        m = 4
    else:
        fam = ws.pendulum_family(8)
        insts = cs.workloads.pendulum_batch(6, K=8, seed=8)
        m = insts[0].m
    solver = ws.BatchSolver(fam)
    N, t, y, z, p, th = ws.pack_family(fam, insts)
    bt = cs.Batch(solver.cp(m), len(insts))
    bt.set_guess_packed(N, t, y, z, p, th)
    bt.solve(solver.opts)
    _check(cs, bt)
    # the files the package writes per instance read back as the solution
    assert ws.write_solution_files(bt, str(tmp_path / "s_%d.data")) == [0] * len(insts)
    for b, s in enumerate(bt.solution()):
        err, t2, y2, z2, p2 = cs.io.bvpdae_read_data(str(tmp_path / ("s_%d.data" % b)))
        assert err == 0
        np.testing.assert_array_equal(y2, s["y"])


def test_device_files_equal_host_writer_on_bit_patterns():
    cs = pkg()
    ws = cs.warmstart
    fam = ws.vdp_family()
    insts = cs.workloads.vdp_batch(12, seed=9, n_range=(32, 64), m_choices=(3,))
    N, t, y, z, p, th = ws.pack_family(fam, insts)
    rng = np.random.default_rng(10)
    y = rng.integers(0, 2**64, y.size, dtype=np.uint64).view(np.float64).reshape(y.shape).copy()
    y.flat[:8] = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -2.5e-310, 1e16]
    p = rng.integers(0, 2**64, p.size, dtype=np.uint64).view(np.float64).reshape(p.shape).copy()
    t = t * np.exp(rng.uniform(-30, 30))
    solver = ws.BatchSolver(fam)
    bt = cs.Batch(solver.cp(3), len(insts))
    bt.set_guess_packed(N, t, y, z, p, th)
    _check(cs, bt)
    # a buffer one byte short is refused (the offsets are still filled)
    off = np.zeros(bt.B + 1, dtype=np.int64)
    assert bt._lib.cs_format_solutions(bt.handle, None, 0, off.ctypes.data) == 0
    buf = np.zeros(int(off[-1]), dtype=np.uint8)
    rc = bt._lib.cs_format_solutions(bt.handle, buf.ctypes.data, int(off[-1]) - 1, off.ctypes.data)
    assert rc == 1 and "too small" in cs._lib.last_error()
