"""Warm-start network kernels (csrc/cs_mlp.cu) against the numpy oracle
(oracle/mlp_oracle.py, same bf16 operand rounding): loss, gradients of every
weight and bias, predictions; and training lowers the loss.

Tolerances: loss 1e-4 relative, gradient vector 2e-3 relative (L2), the
prediction 2e-3 relative (L2) and 1e-2 of the output scale for any entry
(FP32 accumulation on the tensor cores against float64 in the oracle)."""
import numpy as np
import pytest

from conftest import pkg
from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu


def _data(n, n_in, n_out, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-2, 3, (n, n_in)).astype(np.float32)
    W = rng.standard_normal((n_in, n_out))
    Y = (np.sin(X @ W) + 0.1 * X.sum(1, keepdims=True)).astype(np.float32)
    return X, Y


@pytest.mark.parametrize("n,n_in,width,depth,n_out", [(64, 4, 32, 4, 10), (200, 7, 96, 3, 70), (130, 4, 256, 4, 322)])
def test_gradient_matches_oracle(n, n_in, width, depth, n_out):
    cs = pkg()
    net = cs.warmstart.Mlp(n_in, n_out, width=width, depth=depth, seed=3)
    X, Y = _data(n, n_in, n_out, seed=n)
    net.fit_normalization(X, Y)
    loss, g = net.gradient(X, Y)
    xm, xs, ym, ys = (a.astype(np.float64) for a in net.norm)
    ref_loss, ref_g = MO.loss_and_grad(net.params().astype(np.float64), net.sizes, X.astype(np.float64),
                                       Y.astype(np.float64), xm, xs, ym, ys)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    assert np.linalg.norm(g - ref_g) <= 2e-3 * np.linalg.norm(ref_g)
    # every layer's weights and bias individually
    o = 0
    for di, dd in net.sizes:
        for sz in (di * dd, dd):
            a, b = g[o:o + sz], ref_g[o:o + sz]
            assert np.linalg.norm(a - b) <= 5e-3 * max(np.linalg.norm(b), 1e-12)
            o += sz


def test_predict_matches_oracle_and_training_lowers_loss():
    cs = pkg()
    X, Y = _data(2048, 4, 40, seed=1)
    net = cs.warmstart.Mlp(4, 40, width=128, depth=4, seed=5)
    net.fit_normalization(X, Y)
    l0, _ = net.gradient(X, Y)
    net.train(X, Y, epochs=60, batch=256, lr=2e-3, seed=1)
    l1, _ = net.gradient(X, Y)
    assert l1 < 0.2 * l0
    P = net.predict(X[:300])
    xm, xs, ym, ys = (a.astype(np.float64) for a in net.norm)
    ref = MO.predict(net.params().astype(np.float64), net.sizes, X[:300].astype(np.float64), xm, xs, ym, ys)
    # an activation that lands on a bf16 rounding boundary may round the other
    # way in FP32 than in float64: a few entries move by one bf16 step
    assert np.linalg.norm(P - ref) <= 2e-3 * np.linalg.norm(ref)
    assert np.abs(P - ref).max() <= 1e-2 * np.abs(ref).max()


def test_cosine_schedule_plumbing():
    """cs_mlp_set_schedule: a cosine from lr to 1.0 * lr is the constant rate
    (same bits); a decay to 0 trains to different parameters, with a finite
    loss no worse than 1.5x the constant rate's on this short run."""
    cs = pkg()
    X, Y = _data(2048, 4, 40, seed=2)
    nets = []
    for lr_final in (None, 1.0, 0.0):
        net = cs.warmstart.Mlp(4, 40, width=64, depth=3, seed=5)
        net.fit_normalization(X, Y)
        net.train(X, Y, epochs=20, batch=256, lr=2e-3, seed=1, lr_final=lr_final)
        nets.append(net)
    np.testing.assert_array_equal(nets[0].params(), nets[1].params())
    assert not np.array_equal(nets[0].params(), nets[2].params())
    l0, _ = nets[0].gradient(X, Y)
    l2, _ = nets[2].gradient(X, Y)
    assert np.isfinite(l2) and l2 <= 1.5 * l0
