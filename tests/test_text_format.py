"""The library's double-to-text conversion (cs_format_double, host build of
the code the GPU solution-file writer runs) against Python's own
"{}".format, which the reference's writer uses (BVPDAEReadWriteData.py:
337-364): shortest round-trip digits, positional or scientific notation."""
import ctypes

import numpy as np

from conftest import pkg


def _fmt(lib, buf, v):
    n = lib.cs_format_double(v, buf)
    assert 0 < n <= 24
    return buf.raw[:n].decode()


def test_format_double_equals_python_format():
    cs = pkg()
    lib = cs._lib.load()
    buf = ctypes.create_string_buffer(32)
    rng = np.random.default_rng(5)
    special = [0.0, -0.0, float("inf"), -float("inf"), float("nan"), 1.0, -1.0, 0.1, 0.5, 1e-4, 1e-5, 9.999e-5,
               1e16, 9999999999999998.0, 1e15, 1234567890123456.0, 5e-324, 2.2250738585072014e-308,
               2.225073858507201e-308, 1.7976931348623157e308, 2.0**53, 2.0**53 + 2, 123.456, 100.0, 1e22, 1e23,
               0.3, 2 / 3, 1 / 3, 1e-323, 1e308, 1e-310, -2.5e-310]
    vals = special + [2.0**k for k in range(-1074, 1024, 7)] + [10.0**k for k in range(-323, 309, 3)]
    vals += list(rng.standard_normal(20000)) + list(np.exp(rng.uniform(-700, 700, 20000)))
    vals += list(rng.integers(0, 2**64, 40000, dtype=np.uint64).view(np.float64))
    vals += [k / 8 for k in range(-200, 200)] + [float(k) for k in range(-100, 100)]
    bad = [(v, _fmt(lib, buf, float(v)), "{}".format(float(v))) for v in vals
           if _fmt(lib, buf, float(v)) != "{}".format(float(v))]
    assert not bad, bad[:5]
    assert lib.cs_format_double(1.0, None) == -1
