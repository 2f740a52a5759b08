"""Host side of the learned warm start (no GPU): trajectory vectors and their
interpolation back onto a mesh, packed guesses of a family, the seeded
instance generators and the features the network sees."""
import numpy as np

from conftest import pkg


def test_trajectory_vector_layout_and_round_trip():
    cs = pkg()
    ws = cs.warmstart
    T, N, ny, nz, npar = 4.0, 301, 3, 2, 2
    t = np.linspace(0.0, T, N)
    y = np.stack([np.sin(2 * np.pi * t / T), np.cos(t), t / T], axis=1)
    z = np.stack([np.exp(-t), 1.0 + 0.0 * t], axis=1)
    p = np.array([0.5, -2.0])
    v = ws.trajectory_vector(t, y, z, p, T)
    assert v.shape == (ws.N_NODES * (ny + nz) + npar,)
    np.testing.assert_array_equal(v[-npar:], p)
    # node 0 and the last node of the vector are the end values exactly
    ys = v[:ws.N_NODES * ny].reshape(ws.N_NODES, ny)
    np.testing.assert_allclose(ys[0], y[0], rtol=0, atol=1e-15)
    np.testing.assert_allclose(ys[-1], y[-1], rtol=0, atol=1e-15)
    # back onto the mesh: two linear interpolations of a smooth function;
    # the error is bounded by h^2/8 max|y''| on the 64-node grid (h = T/63)
    y2, z2, p2 = ws.guess_from_vector(v, t, T, ny, nz, npar)
    h = T / (ws.N_NODES - 1)
    bound = 2 * h * h / 8 * max((2 * np.pi / T) ** 2, 1.0)
    assert np.abs(y2 - y).max() <= bound
    assert np.abs(z2 - z).max() <= bound
    np.testing.assert_array_equal(p2, p)


def test_trajectory_vector_of_a_linear_trajectory_is_exact():
    """Linear interpolation reproduces a linear trajectory on any mesh."""
    cs = pkg()
    ws = cs.warmstart
    T = 7.5
    t = np.sort(np.concatenate([[0.0, T], np.random.default_rng(3).uniform(0, T, 40)]))
    y = np.stack([2.0 - 0.3 * t, 0.1 * t], axis=1)
    z = (1.0 + t)[:, None]
    v = ws.trajectory_vector(t, y, z, np.zeros(0), T)
    y2, z2, _ = ws.guess_from_vector(v, np.linspace(0.0, T, 17), T, 2, 1, 0)
    tt = np.linspace(0.0, T, 17)
    np.testing.assert_allclose(y2, np.stack([2.0 - 0.3 * tt, 0.1 * tt], axis=1), rtol=0, atol=1e-12)
    np.testing.assert_allclose(z2[:, 0], 1.0 + tt, rtol=0, atol=1e-12)


def test_pack_family_matches_the_instances():
    cs = pkg()
    ws = cs.warmstart
    fam = ws.vdp_family()
    insts = cs.workloads.vdp_batch(7, seed=4, n_range=(10, 40))
    N, t, y, z, p, th = ws.pack_family(fam, insts)
    assert N.dtype == np.int32 and list(N) == [i.intervals + 1 for i in insts]
    assert t.shape == (N.sum(),) and y.shape == (N.sum(), fam.ny) and z.shape == (N.sum(), fam.nz)
    assert p.shape == (7, fam.np) and th.shape == (7, 3)
    o = 0
    for k, inst in enumerate(insts):
        tk = t[o:o + N[k]]
        assert tk[0] == 0.0 and tk[-1] == inst.T and np.all(np.diff(tk) > 0)
        np.testing.assert_array_equal(th[k], inst.theta)
        o += N[k]
    assert fam.n_out == ws.N_NODES * (fam.ny + fam.nz) + fam.np
    assert fam.features(insts[0]).shape == (4,)


def test_instance_generators_are_seeded_and_in_range():
    cs = pkg()
    w = cs.workloads
    a = w.vdp_batch(500, seed=9)
    b = w.vdp_batch(500, seed=9)
    assert all((x.x0 == y.x0).all() and (x.T, x.r, x.intervals, x.m) == (y.T, y.r, y.intervals, y.m)
               for x, y in zip(a, b))
    assert all(-2 <= i.x0.min() and i.x0.max() <= 2 for i in a)
    assert all(2.0 <= i.T <= 8.0 and 0.1 <= i.r <= 10.0 and 32 <= i.intervals <= 2048 for i in a)
    assert {i.m for i in a} == {3, 4, 5}
    c = w.vdp_batch(500, seed=10)
    assert any(x.T != y.T for x, y in zip(a, c))
    pend = w.pendulum_batch(50, K=8, seed=2)
    assert all(i.theta0.shape == (8,) and np.abs(i.theta0).max() <= 0.5 for i in pend)
    assert all(5.0 <= i.T <= 15.0 and 0.2 <= i.k <= 1.0 and 32 <= i.intervals <= 128 and i.m == 4 for i in pend)


def test_pendulum_plain_guess_is_the_linear_decay():
    """theta_i(t) = theta_i(0) (1 - t/T), every other value 0, p = 1."""
    cs = pkg()
    inst = cs.workloads.pendulum_batch(1, K=4, seed=5)[0]
    t, y, z, p = inst.guess(10, 1, 6)
    assert t[0] == 0.0 and t[-1] == inst.T and len(t) == inst.intervals + 1
    np.testing.assert_allclose(y[:, :4], inst.theta0[None, :] * (1.0 - t / inst.T)[:, None], rtol=0, atol=1e-15)
    assert not y[:, 4:].any() and not z.any()
    np.testing.assert_array_equal(p, np.ones(6))
    np.testing.assert_array_equal(inst.theta, np.concatenate([[inst.k], inst.theta0]))
