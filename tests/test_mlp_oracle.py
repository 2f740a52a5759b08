"""The MLP oracle's analytic gradient against central finite differences
(bf16 rounding switched off for the check), and the bf16 rounding rule."""
import numpy as np

from conftest import pkg
from oracle import mlp_oracle as MO


def test_oracle_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(MO, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(0)
    sizes = [(3, 8), (8, 8), (8, 8), (8, 5)]
    npar = sum(a * b + b for a, b in sizes)
    p = rng.standard_normal(npar) * 0.5
    X, Y = rng.standard_normal((20, 3)), rng.standard_normal((20, 5))
    args = (np.zeros(3), np.ones(3), np.zeros(5), np.ones(5))
    _, g = MO.loss_and_grad(p, sizes, X, Y, *args)
    fd = np.zeros(npar)
    for k in range(npar):
        e = np.zeros(npar)
        e[k] = 1e-6
        fd[k] = (MO.loss_and_grad(p + e, sizes, X, Y, *args)[0] - MO.loss_and_grad(p - e, sizes, X, Y, *args)[0]) / 2e-6
    assert np.linalg.norm(fd - g) <= 1e-6 * np.linalg.norm(g)


def test_bf16_rounds_to_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.0 - 2 ** -7 - 2 ** -9, 3.14159265], dtype=np.float64)
    np.testing.assert_array_equal(MO.bf16(v), [1.0, 1.0, 1.0 + 2 ** -6, -2.0 - 2 ** -6, 3.140625])


def test_trajectory_round_trip():
    cs = pkg()
    ws = cs.warmstart
    t = np.linspace(0, 3.0, 201)
    y = np.stack([np.sin(t), np.cos(t)], axis=1)
    z = t[:, None] ** 2
    v = ws.trajectory_vector(t, y, z, [0.5, -1.0], 3.0)
    y2, z2, p2 = ws.guess_from_vector(v, t, 3.0, 2, 1, 2)
    assert np.abs(y2 - y).max() < 2e-3 and np.abs(z2 - z).max() < 2e-3
    np.testing.assert_array_equal(p2, [0.5, -1.0])
