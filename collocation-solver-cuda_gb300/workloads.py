"""Seeded synthetic instance families (no public dataset is involved).

vdp_batch       Van der Pol family: x0 ~ U[-2,2]^2, T ~ U[2,8], control weight
                r ~ logU[0.1,10], N ~ integer U[32,2048] intervals, m uniform in
                {3,4,5}, zero initial guess (costates and control zero, the
                kappa multipliers start at 1 as the reference's generated
                BvpDae does), tol 1e-6.
pendulum_ocp    OCP text of a chain of K pendulums (coupling k, free ends,
                every 4th pendulum actuated, cost |theta|^2 + |theta'|^2 +
                0.1 |u|^2 on [0, T]); initial angles are instance constants.
pendulum_chain_problem
                the single large instances: K = 16 (Nodes 8193, m = 5,
                tol 1e-6, theta(0) seed 0) and K = 32 (Nodes 16385, m = 4,
                tol 1e-8, seed 2).
"""
import os

import numpy as np

from .ocp import Problem

HERE = os.path.dirname(os.path.abspath(__file__))

VDP_FAMILY_OCP = os.path.join(HERE, "problems", "vdp_family.ocp")


def vdp_family_problem(max_nodes=20000):
    pr = Problem.from_file(VDP_FAMILY_OCP)
    pr.maximum_nodes = max_nodes
    return pr


class VdpInstance:
    __slots__ = ("x0", "T", "r", "intervals", "m")

    def __init__(self, x0, T, r, intervals, m):
        self.x0, self.T, self.r, self.intervals, self.m = x0, T, r, intervals, m

    @property
    def theta(self):
        return np.array([self.x0[0], self.x0[1], self.r])

    def guess(self, ny=4, nz=1, np_=2):
        N = self.intervals + 1
        t = np.linspace(0.0, self.T, N)
        return t, np.zeros((N, ny)), np.zeros((N, nz)), np.ones(np_)


def vdp_batch(n, seed=1, n_range=(32, 2048), m_choices=(3, 4, 5), x0_range=2.0, T_range=(2.0, 8.0),
              r_range=(0.1, 10.0)):
    """n instances of the Van der Pol family, seeded."""
    rng = np.random.default_rng(seed)
    x0 = rng.uniform(-x0_range, x0_range, (n, 2))
    T = rng.uniform(T_range[0], T_range[1], n)
    r = np.exp(rng.uniform(np.log(r_range[0]), np.log(r_range[1]), n))
    N = rng.integers(n_range[0], n_range[1] + 1, n)
    m = rng.choice(np.array(m_choices), n)
    return [VdpInstance(x0[i], float(T[i]), float(r[i]), int(N[i]), int(m[i])) for i in range(n)]


def pack_vdp(instances, ny=4, nz=1, np_=2):
    """Packed host arrays (N, t, y, z, p, theta) for a list of instances."""
    Ns = np.array([inst.intervals + 1 for inst in instances], dtype=np.int32)
    T = int(Ns.sum())
    t = np.zeros(T)
    o = 0
    for inst, n in zip(instances, Ns):
        t[o:o + n] = np.linspace(0.0, inst.T, n)
        o += n
    y = np.zeros((T, ny))
    z = np.zeros((T, nz))
    p = np.ones((len(instances), np_))
    th = np.array([inst.theta for inst in instances])
    return Ns, t, y, z, p, th


class PendulumInstance:
    """One instance of the pendulum-chain family: initial angles theta0 (K),
    final time T, coupling k, mesh intervals and m."""
    __slots__ = ("theta0", "T", "k", "intervals", "m")

    def __init__(self, theta0, T, k, intervals, m):
        self.theta0, self.T, self.k, self.intervals, self.m = theta0, T, k, intervals, m

    @property
    def theta(self):
        """Instance constants in the OCP's order: kc, a1 .. aK."""
        return np.concatenate([[self.k], self.theta0])

    def guess(self, ny, nz, np_):
        """theta_i(t) = theta_i(0) (1 - t/T), every other value 0, p = 1."""
        N = self.intervals + 1
        t = np.linspace(0.0, self.T, N)
        y = np.zeros((N, ny))
        K = len(self.theta0)
        y[:, :K] = self.theta0[None, :] * (1.0 - t / self.T)[:, None]
        return t, y, np.zeros((N, nz)), np.ones(np_)


def pendulum_family_problem(K=8, max_nodes=20000):
    """The pendulum chain with kc and the initial angles as instance
    constants (the final time comes from each instance's mesh)."""
    pr = Problem(pendulum_ocp(K, np.zeros(K), max_nodes=max_nodes), name="pendulum%d_family" % K)
    pr.maximum_nodes = max_nodes
    return pr


def pendulum_batch(n, K=8, seed=1, n_range=(32, 128), m_choices=(4,), theta_range=0.5, T_range=(5.0, 15.0),
                   k_range=(0.2, 1.0)):
    """n seeded instances of the pendulum-chain family: theta(0) ~ U[-0.5,0.5]^K,
    T ~ U[5,15], coupling k ~ U[0.2,1.0]."""
    rng = np.random.default_rng(seed)
    th = rng.uniform(-theta_range, theta_range, (n, K))
    T = rng.uniform(T_range[0], T_range[1], n)
    k = rng.uniform(k_range[0], k_range[1], n)
    N = rng.integers(n_range[0], n_range[1] + 1, n)
    m = rng.choice(np.array(m_choices), n)
    return [PendulumInstance(th[i], float(T[i]), float(k[i]), int(N[i]), int(m[i])) for i in range(n)]


def pendulum_ocp(K, theta0, T=10.0, k=0.5, nodes=101, actuated_every=4, ctrl_weight=0.1, tol=1e-6,
                 max_nodes=40000):
    """OCP text for a chain of K pendulums with free ends."""
    th = ["th%d" % (i + 1) for i in range(K)]
    w = ["w%d" % (i + 1) for i in range(K)]
    act = list(range(0, K, actuated_every))
    us = ["u%d" % (j + 1) for j in range(len(act))]
    consts = ["kc = %r" % float(k)] + ["a%d = %r" % (i + 1, float(theta0[i])) for i in range(K)]
    dyn = []
    for i in range(K):
        left = th[i - 1] if i > 0 else th[i]
        right = th[i + 1] if i < K - 1 else th[i]
        e = "-sin(%s) + kc*(%s - 2.0*%s + %s)" % (th[i], right, th[i], left)
        if i in act:
            e += " + " + us[act.index(i)]
        dyn.append(e)
    cost = "0.5*(" + " + ".join("%s*%s" % (v, v) for v in th + w) + " + %r*(" % ctrl_weight + \
        " + ".join("%s*%s" % (u, u) for u in us) + "))"
    est = ["a%d*(1.0 - t/%r)" % (i + 1, float(T)) for i in range(K)] + ["0.0"] * (3 * K)
    lines = [
        "Constants = [%s];" % ", ".join(consts),
        "StateVariables = [%s];" % ", ".join(th + w),
        "ControlVariables = [%s];" % ", ".join(us),
        "InitialConstraints = [%s];" % ", ".join(["%s - a%d" % (th[i], i + 1) for i in range(K)] + w),
        "CostFunctional = %s;" % cost,
        "DifferentialEquations = [%s];" % ", ".join(w + dyn),
        "InitialTime = 0.0;",
        "FinalTime = %r;" % float(T),
        "Nodes = %d;" % nodes,
        "Tolerance = %r;" % tol,
        "MaximumNodes = %d;" % max_nodes,
        "StateEstimate = [%s];" % ", ".join(est),
        "ControlEstimate = [%s];" % ", ".join(["0.0"] * len(us)),
        'OutputFile = "pendulum%d.data";' % K,
    ]
    return "\n".join(lines) + "\n"


# the single large instances: chain length K -> collocation points, nodes,
# tolerance and the seed of theta(0) ~ U[-0.5, 0.5]^K
PENDULUM_CHAINS = {16: dict(m=5, nodes=8193, tol=1e-6, seed=0), 32: dict(m=4, nodes=16385, tol=1e-8, seed=2)}


def pendulum_chain_problem(K, nodes=None):
    """The large pendulum-chain instance of length K (16 or 32) with its
    initial guess theta_i(t) = theta_i(0) (1 - t/T), other values 0, on a
    uniform mesh of `nodes` (default: the stated size)."""
    c = PENDULUM_CHAINS[K]
    theta0 = np.random.default_rng(c["seed"]).uniform(-0.5, 0.5, K)
    return Problem(pendulum_ocp(K, theta0, nodes=nodes or c["nodes"], tol=c["tol"]), name="pend%d" % K)
