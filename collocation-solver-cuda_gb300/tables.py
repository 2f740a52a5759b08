"""Quadrature and collocation tables, computed from their definitions.

Lobatto IIIA (m stages, m = 3..10) on [0, 1]:
    c_j  : the Gauss-Lobatto points, 0, 1 and the roots of P'_{m-1}(2c - 1)
    A_jk : integral over [0, c_j] of the k-th Lagrange basis polynomial on c
    b_k  : integral over [0, 1] of the same polynomial
Gauss-Legendre (n points) on [0, 1]: nodes and weights.

The reference stores these as literal tables (collocation_coefficients.py:10-637
for Lobatto A, b, c; gauss_coefficients.py:6-131 for Gauss points) and writes
the Lagrange basis L_k(t) and its integral I_k(t) as polynomials with truncated
15-digit coefficients (collocation_coefficients.py:638-788).  Here every value
is evaluated in 50-digit arithmetic and rounded once to float64, so the tables
agree with the reference's to the rounding of its literals (about 1e-15).
"""
import functools

import mpmath
import numpy as np

_DPS = 50


def _lobatto_nodes_mp(m):
    """Gauss-Lobatto nodes on [0, 1] as mpf, ascending."""
    with mpmath.workdps(_DPS):
        if m < 2:
            raise ValueError("Lobatto collocation needs m >= 2")
        # interior nodes: roots of d/dx P_{m-1}(x) on (-1, 1)
        n = m - 1
        coeffs = mpmath.taylor(lambda x: mpmath.diff(lambda s: mpmath.legendre(n, s), x), 0, n - 1)
        coeffs = [mpmath.mpf(c) for c in coeffs]
        interior = []
        if n - 1 >= 1:
            interior = sorted(mpmath.re(r) for r in mpmath.polyroots(coeffs[::-1], maxsteps=200, extraprec=200))
        xs = [mpmath.mpf(-1)] + interior + [mpmath.mpf(1)]
        return [(x + 1) / 2 for x in xs]


def _lagrange_poly_mp(nodes, k):
    """Coefficients (ascending powers) of the k-th Lagrange basis polynomial."""
    with mpmath.workdps(_DPS):
        poly = [mpmath.mpf(1)]
        denom = mpmath.mpf(1)
        for j, xj in enumerate(nodes):
            if j == k:
                continue
            # multiply by (t - xj)
            new = [mpmath.mpf(0)] * (len(poly) + 1)
            for i, a in enumerate(poly):
                new[i] -= a * xj
                new[i + 1] += a
            poly = new
            denom *= (nodes[k] - xj)
        return [a / denom for a in poly]


def _polyval_mp(coeffs, t):
    acc = mpmath.mpf(0)
    for a in reversed(coeffs):
        acc = acc * t + a
    return acc


def _polyint_mp(coeffs, t):
    """Integral from 0 to t."""
    acc = mpmath.mpf(0)
    for i in range(len(coeffs) - 1, -1, -1):
        acc = acc * t + coeffs[i] / (i + 1)
    return acc * t


class Lobatto:
    """Lobatto IIIA tableau with A (m x m), b (m), c (m) in float64."""

    def __init__(self, m):
        self.m = m
        with mpmath.workdps(_DPS):
            c = _lobatto_nodes_mp(m)
            polys = [_lagrange_poly_mp(c, k) for k in range(m)]
            self.A = np.array([[float(_polyint_mp(polys[k], c[j])) for k in range(m)] for j in range(m)])
            self.b = np.array([float(_polyint_mp(polys[k], mpmath.mpf(1))) for k in range(m)])
            self.c = np.array([float(x) for x in c])
        self.c[0] = 0.0
        self.c[-1] = 1.0
        self.A[0, :] = 0.0
        self._nodes_mp = c
        self._polys = polys

    def basis(self, t):
        """L_k(t) for k = 0..m-1 (Lagrange basis on the collocation points)."""
        with mpmath.workdps(_DPS):
            tt = mpmath.mpf(t)
            return np.array([float(_polyval_mp(p, tt)) for p in self._polys])

    def basis_integral(self, t):
        """I_k(t) = integral_0^t L_k for k = 0..m-1."""
        with mpmath.workdps(_DPS):
            tt = mpmath.mpf(t)
            return np.array([float(_polyint_mp(p, tt)) for p in self._polys])


class Gauss:
    """n-point Gauss-Legendre rule on [0, 1]: nodes t, weights w (float64)."""

    def __init__(self, n):
        self.n = n
        with mpmath.workdps(_DPS):
            xs = sorted(mpmath.polyroots(_legendre_coeffs(n)[::-1], maxsteps=200, extraprec=200), key=lambda v: mpmath.re(v))
            xs = [mpmath.re(x) for x in xs]
            ws = []
            for x in xs:
                dp = mpmath.diff(lambda s: mpmath.legendre(n, s), x)
                ws.append(2 / ((1 - x * x) * dp * dp))
            self._t_mp = [(x + 1) / 2 for x in xs]
            self.t = np.array([float(v) for v in self._t_mp])
            self.w = np.array([float(v / 2) for v in ws])


def _legendre_coeffs(n):
    with mpmath.workdps(_DPS):
        return [mpmath.mpf(c) for c in mpmath.taylor(lambda s: mpmath.legendre(n, s), 0, n)]


@functools.lru_cache(maxsize=None)
def lobatto(m):
    return Lobatto(m)


@functools.lru_cache(maxsize=None)
def gauss(n):
    return Gauss(n)


@functools.lru_cache(maxsize=None)
def segment_tables(m):
    """Tables the mesh-error pass needs for m collocation points: Gauss nodes and
    weights of the (m+1)-point rule, the basis L_k and its integral I_k at those
    nodes (shape (m+1, m)), and L_k at t = 0 and t = 1 (node recovery)."""
    lo = lobatto(m)
    g = gauss(m + 1)
    with mpmath.workdps(_DPS):
        L = np.array([[float(_polyval_mp(p, t)) for p in lo._polys] for t in g._t_mp])
        I = np.array([[float(_polyint_mp(p, t)) for p in lo._polys] for t in g._t_mp])
    L0 = lo.basis(0)
    L1 = lo.basis(1)
    return dict(tau=g.t.copy(), w=g.w.copy(), L=L, I=I, L0=L0, L1=L1)
