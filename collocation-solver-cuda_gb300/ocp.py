"""Front end: the plain-text OCP format -> Pontryagin BVP-DAE (sympy).

The input format is the reference's (OCP2ABVP.py:472-793): statements end with
';', '#' starts a comment, whitespace is ignored, and each statement starts
with a keyword (Constants, Variables, StateVariables, ControlVariables,
ParameterVariables, TerminalPenalty, CostFunctional, InitialConstraints,
TerminalConstraints, DifferentialEquations, InequalityConstraints,
StateVariableInequalityConstraints, EqualityConstraints, InitialTime,
FinalTime, Nodes, Tolerance, InputFile, OutputFile, Display,
MaximumMeshRefinements, MaximumNewtonIterations, MaximumNodes,
StateEstimate, ControlEstimate, ParameterEstimate) or is the definition
`name = expr;` of a name listed in `Variables`, which is then substituted,
parenthesised, wherever it appears in later expressions.

Expressions are evaluated with Python semantics over sympy symbols, as the
reference does, so literals such as `1/2` are Python floats.

The derivation (OCP2ABVP.py:41-182) produces, with n_x states, n_u controls,
n_c equality, n_d inequality and n_s state-inequality constraints:

    y = [x, lambda, gamma]                     (2 n_x + n_p)
    z = [u, theta, mu, xi, nu, sigma]          (n_u + n_c + 2 n_d + 2 n_s)
    p = [p, kappa_i, kappa_f]                  (n_p + n_Gamma + n_Psi)
    H = L + lambda.f (+ alpha |u|^2 / 2 if n_d + n_s > 0)
          + theta.c + mu.d + xi.s
    y' = [H_lambda, -H_x, H_p]
    0  = [H_u, H_theta, H_mu + nu - alpha mu, H_xi + sigma - alpha xi,
          mu + nu - sqrt(mu^2 + nu^2 + 2 alpha), xi + sigma - sqrt(xi^2 + sigma^2 + 2 alpha)]
    0  = r(y(t0), y(tf), p) = [Gamma; lambda + Gamma_x kappa_i; gamma]  at t0
                              [Psi; lambda - phi_x - Psi_x kappa_f; gamma + phi_p + Psi_p kappa_f] at tf

The symbol order, the signs of the boundary conditions and the smoothed
Fischer-Burmeister terms are kept exactly so that the unknown vector and the
residual match the reference's generated bvp_problem.py element for element.

Every `Constants` entry stays symbolic in f, g and r and becomes a slot of the
per-instance constant vector theta (default: the value in the file).  This is
what lets one compiled module solve a batch of instances that differ only in
constants.
"""
import math
import re

import numpy as np
import sympy

_KEYWORDS = [
    # order matters where one keyword is a prefix of another
    "Constants", "StateVariables", "ControlVariables", "ParameterVariables", "TerminalPenalty",
    "CostFunctional", "InitialConstraints", "TerminalConstraints", "DifferentialEquations",
    "InequalityConstraints", "StateVariableInequalityConstraints", "EqualityConstraints",
    "InitialTime", "FinalTime", "Nodes", "Tolerance", "InputFile", "OutputFile", "Display",
    "MaximumMeshRefinements", "MaximumNewtonIterations", "MaximumNodes", "StateEstimate",
    "ControlEstimate", "ParameterEstimate", "Variables",
]


class OcpSyntaxError(SyntaxError):
    pass


def _statements(text):
    """Comment-stripped, whitespace-free statements, each ending at ';'."""
    out = []
    cur = []
    for raw in text.splitlines(True):
        line = raw.split("#", 1)[0]
        for ch in line:
            if ch in "\n\r\t ":
                continue
            cur.append(ch)
            if ch == ";":
                out.append("".join(cur))
                cur = []
    return out


def _bracket_items(stmt):
    """Items of `Keyword=[a,b,c];` (top-level commas only)."""
    i = stmt.find("[")
    j = stmt.rfind("]")
    if i < 0 or j < i:
        raise OcpSyntaxError("expected [...] in: %s" % stmt)
    body = stmt[i + 1:j]
    items, depth, cur = [], 0, []
    for ch in body:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            items.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    if cur or items:
        items.append("".join(cur))
    return items


def _rhs(stmt):
    i = stmt.find("=")
    if i < 0:
        raise OcpSyntaxError("expected '=' in: %s" % stmt)
    return stmt[i + 1:].rstrip(";")


def _is_ident_char(ch):
    return ch.isalnum() or ch == "_"


def _substitute_word(expr, name, replacement):
    """Replace whole-word occurrences of `name` in `expr`."""
    out = []
    i = 0
    n = len(name)
    while i < len(expr):
        if expr.startswith(name, i) and (i == 0 or not _is_ident_char(expr[i - 1])) and \
                (i + n >= len(expr) or not _is_ident_char(expr[i + n])):
            out.append(replacement)
            i += n
        else:
            out.append(expr[i])
            i += 1
    return "".join(out)


class OcpSpec:
    """Parsed OCP text (still symbolic)."""

    def __init__(self):
        self.constants = []          # names
        self.constant_values = []    # float
        self.constant_exprs = []     # value strings as written
        self.x, self.u, self.p = [], [], []
        self.phi = sympy.Integer(0)
        self.L = sympy.Integer(0)
        self.f, self.c, self.d, self.s = [], [], [], []
        self.Gamma, self.Psi = [], []
        self.t_i, self.t_f = 0, 1
        self.nodes = 100
        self.input_file = ""
        self.output_file = "ocp.data"
        self.tolerance = 1.0e-6
        self.maximum_nodes = 2000
        self.maximum_newton_iterations = 200
        self.maximum_mesh_refinements = 10
        self.display = 0
        self.state_estimate = None
        self.control_estimate = None
        self.parameter_estimate = None
        self.source = ""


def _namespace(spec):
    ns = {}
    exec("from sympy import *", ns)  # sympy's public names, as the reference's exec scope
    ns["NO"], ns["YES"] = 0, 1
    ns["t"] = sympy.Symbol("t")
    for name in spec.constants:
        ns[name] = sympy.Symbol(name)
    for name in spec.x + spec.u + spec.p:
        ns[name] = sympy.Symbol(name)
    return ns


def parse_ocp(text):
    """Parse OCP text into an OcpSpec (raises OcpSyntaxError)."""
    spec = OcpSpec()
    spec.source = text
    stmts = _statements(text)
    # pass 1: Variables macros
    macro_names = []
    for st in stmts:
        if st.startswith("Variables"):
            macro_names = [v for v in _bracket_items(st) if v]
    macros = {}
    for st in stmts:
        for v in macro_names:
            if st.startswith(v + "="):
                macros[v] = "(" + st[len(v) + 1:].rstrip(";") + ")"

    def expand(expr, depth=0):
        if depth > 50:
            raise OcpSyntaxError("recursive Variables definition")
        changed = True
        while changed:
            changed = False
            for v, body in macros.items():
                new = _substitute_word(expr, v, body)
                if new != expr:
                    expr = new
                    changed = True
            depth += 1
            if depth > 50:
                raise OcpSyntaxError("recursive Variables definition")
        return expr

    ns = None

    def ev(expr):
        nonlocal ns
        if ns is None:
            ns = _namespace(spec)
        try:
            return eval(expand(expr), dict(ns))
        except Exception as e:  # noqa: BLE001
            raise OcpSyntaxError("cannot evaluate '%s': %s" % (expr, e))

    def ev_list(st):
        return [ev(item) for item in _bracket_items(st)]

    def literal(st):
        v = _rhs(st)
        try:
            return eval(v, {"NO": 0, "YES": 1, "__builtins__": {}})
        except Exception as e:  # noqa: BLE001
            raise OcpSyntaxError("bad value in '%s': %s" % (st, e))

    for st in stmts:
        kw = None
        for k in _KEYWORDS:
            if st.startswith(k):
                kw = k
                break
        if kw is None:
            if any(st.startswith(v + "=") for v in macro_names):
                continue
            raise OcpSyntaxError("unknown statement: %s" % st)
        if kw == "Constants":
            for item in _bracket_items(st):
                name, val = item.split("=", 1)
                spec.constants.append(name)
                spec.constant_exprs.append(val)
                spec.constant_values.append(float(eval(val, {"__builtins__": {}}, {k: getattr(math, k) for k in dir(math) if not k.startswith("_")})))
            ns = None
        elif kw in ("StateVariables", "ControlVariables", "ParameterVariables"):
            names = [v for v in _bracket_items(st) if v]
            {"StateVariables": spec.x, "ControlVariables": spec.u, "ParameterVariables": spec.p}[kw][:] = names
            ns = None
        elif kw == "TerminalPenalty":
            spec.phi = sympy.sympify(ev(_rhs(st)))
        elif kw == "CostFunctional":
            spec.L = sympy.sympify(ev(_rhs(st)))
        elif kw == "InitialConstraints":
            spec.Gamma = [sympy.sympify(e) for e in ev_list(st)]
        elif kw == "TerminalConstraints":
            spec.Psi = [sympy.sympify(e) for e in ev_list(st)]
        elif kw == "DifferentialEquations":
            spec.f = [sympy.sympify(e) for e in ev_list(st)]
        elif kw == "InequalityConstraints":
            spec.d = [sympy.sympify(e) for e in ev_list(st)]
        elif kw == "StateVariableInequalityConstraints":
            spec.s = [sympy.sympify(e) for e in ev_list(st)]
        elif kw == "EqualityConstraints":
            spec.c = [sympy.sympify(e) for e in ev_list(st)]
        elif kw == "InitialTime":
            spec.t_i = literal(st)
        elif kw == "FinalTime":
            spec.t_f = literal(st)
        elif kw == "Nodes":
            spec.nodes = int(literal(st))
        elif kw == "Tolerance":
            spec.tolerance = float(literal(st))
        elif kw == "InputFile":
            spec.input_file = literal(st)
        elif kw == "OutputFile":
            spec.output_file = literal(st)
        elif kw == "Display":
            spec.display = literal(st)
        elif kw == "MaximumMeshRefinements":
            spec.maximum_mesh_refinements = int(literal(st))
        elif kw == "MaximumNewtonIterations":
            spec.maximum_newton_iterations = int(literal(st))
        elif kw == "MaximumNodes":
            spec.maximum_nodes = int(literal(st))
        elif kw in ("StateEstimate", "ControlEstimate", "ParameterEstimate"):
            vals = ev_list(st)
            setattr(spec, {"StateEstimate": "state_estimate", "ControlEstimate": "control_estimate",
                           "ParameterEstimate": "parameter_estimate"}[kw], vals)
        elif kw == "Variables":
            pass
    if len(spec.f) != len(spec.x):
        raise OcpSyntaxError("DifferentialEquations has %d entries for %d states" % (len(spec.f), len(spec.x)))
    return spec


class BvpDaeSymbolic:
    """The Pontryagin BVP-DAE of an OCP, still symbolic."""

    def __init__(self, spec):
        self.spec = spec
        o = spec
        S = sympy.Symbol
        nx, npar = len(o.x), len(o.p)
        nu, nc, nd, ns = len(o.u), len(o.c), len(o.d), len(o.s)
        xs = [S(v) for v in o.x]
        us = [S(v) for v in o.u]
        ps = [S(v) for v in o.p]
        lam = [S("_lambda%d" % (i + 1)) for i in range(nx)]
        gam = [S("_gamma%d" % (i + 1)) for i in range(npar)]
        self.y = xs + lam + gam
        theta = [S("_theta%d" % (i + 1)) for i in range(nc)]
        mu = [S("_mu%d" % (i + 1)) for i in range(nd)]
        xi = [S("_xi%d" % (i + 1)) for i in range(ns)]
        nuv = [S("_nu%d" % (i + 1)) for i in range(nd)]
        sig = [S("_sigma%d" % (i + 1)) for i in range(ns)]
        self.z = us + theta + mu + xi + nuv + sig
        kap_i = [S("_kappa_i%d" % (i + 1)) for i in range(len(o.Gamma))]
        kap_f = [S("_kappa_f%d" % (i + 1)) for i in range(len(o.Psi))]
        self.p = ps + kap_i + kap_f
        alpha = S("_alpha")
        self.alpha = alpha
        self.theta = [S(c) for c in o.constants]

        H = o.L
        for i in range(nx):
            H = H + lam[i] * o.f[i]
        if nd > 0 or ns > 0:
            for ui in us:
                H = H + alpha * ui * ui / 2
        for i in range(nc):
            H = H + theta[i] * o.c[i]
        for i in range(nd):
            H = H + mu[i] * o.d[i]
        for i in range(ns):
            H = H + xi[i] * o.s[i]
        self.H = H

        f = [sympy.diff(H, lam[i]) for i in range(nx)] + [-sympy.diff(H, xs[i]) for i in range(nx)] + \
            [sympy.diff(H, ps[i]) for i in range(npar)]
        g = [sympy.Integer(0)] * len(self.z)
        for i in range(nu):
            g[i] = sympy.diff(H, us[i])
        for i in range(nc):
            g[nu + i] = sympy.diff(H, theta[i])
        for i in range(nd):
            g[nu + nc + i] = sympy.diff(H, mu[i]) + nuv[i] - alpha * mu[i]
            g[nu + nc + nd + ns + i] = mu[i] + nuv[i] - sympy.sqrt(mu[i] ** 2 + nuv[i] ** 2 + 2 * alpha)
        for i in range(ns):
            g[nu + nc + nd + i] = sympy.diff(H, xi[i]) + sig[i] - alpha * xi[i]
            g[nu + nc + nd + ns + nd + i] = xi[i] + sig[i] - sympy.sqrt(xi[i] ** 2 + sig[i] ** 2 + 2 * alpha)
        self.f = [sympy.sympify(e) for e in f]
        self.g = [sympy.sympify(e) for e in g]

        ng, npsi = len(o.Gamma), len(o.Psi)
        ri = list(o.Gamma)
        for i in range(nx):
            acc = sympy.Integer(0)
            for j in range(ng):
                acc += sympy.diff(o.Gamma[j], xs[i]) * kap_i[j]
            ri.append(lam[i] + acc)
        for i in range(npar):
            ri.append(gam[i])
        rf = list(o.Psi)
        for i in range(nx):
            acc = sympy.Integer(0)
            for j in range(npsi):
                acc += sympy.diff(o.Psi[j], xs[i]) * kap_f[j]
            rf.append(lam[i] - sympy.diff(o.phi, xs[i]) - acc)
        for i in range(npar):
            acc = sympy.Integer(0)
            for j in range(npsi):
                acc += sympy.diff(o.Psi[j], ps[i]) * kap_f[j]
            rf.append(gam[i] + sympy.diff(o.phi, ps[i]) + acc)
        self.ri = [sympy.sympify(e) for e in ri]
        self.rf = [sympy.sympify(e) for e in rf]

        self.ny, self.nz, self.np = len(self.y), len(self.z), len(self.p)
        self.n_ineq, self.n_svineq = nd, ns
        if len(self.ri) + len(self.rf) != self.ny + self.np:
            raise OcpSyntaxError("boundary conditions: %d + %d equations for %d unknowns"
                                 % (len(self.ri), len(self.rf), self.ny + self.np))
        # parameters that f or g depend on: only these give nonzero V columns
        used = set()
        for e in self.f + self.g:
            used |= e.free_symbols
        self.p_used = [i for i, s in enumerate(self.p) if s in used]
        self.np_eff = (max(self.p_used) + 1) if self.p_used else 0

    # -- derivative blocks (rows x columns over [y, z, p]) --
    def jac_fg(self):
        cols = self.y + self.z + self.p
        Df = [[sympy.diff(e, v) for v in cols] for e in self.f]
        Dg = [[sympy.diff(e, v) for v in cols] for e in self.g]
        return Df, Dg

    def bc_exprs(self):
        """r as expressions of y0-, y1- and p-symbols; Dr over [y0, y1, p]."""
        y0 = [sympy.Symbol("_y0_%d" % i) for i in range(self.ny)]
        y1 = [sympy.Symbol("_y1_%d" % i) for i in range(self.ny)]
        s0 = dict(zip(self.y, y0))
        s1 = dict(zip(self.y, y1))
        r = [e.xreplace(s0) for e in self.ri] + [e.xreplace(s1) for e in self.rf]
        cols = y0 + y1 + self.p
        Dr = [[sympy.diff(e, v) for v in cols] for e in r]
        return y0, y1, r, Dr


class Problem:
    """A parsed and derived OCP with the reference's BvpDae attributes
    (OCP2ABVP.py:330-447): size_y/z/p, size_inequality, size_sv_inequality,
    output_file, tolerance, maximum_nodes, maximum_newton_iterations,
    maximum_mesh_refinements, N, T0, Y0, Z0, P0, plus `theta` (constant values).
    """

    def __init__(self, text, name="ocp", base_dir=None):
        self.name = name
        self.spec = parse_ocp(text)
        self.sym = BvpDaeSymbolic(self.spec)
        s, o = self.sym, self.spec
        self.size_y, self.size_z, self.size_p = s.ny, s.nz, s.np
        self.size_inequality, self.size_sv_inequality = s.n_ineq, s.n_svineq
        self.output_file = o.output_file
        self.tolerance = o.tolerance
        self.maximum_nodes = o.maximum_nodes
        self.maximum_newton_iterations = o.maximum_newton_iterations
        self.maximum_mesh_refinements = o.maximum_mesh_refinements
        self.theta = np.array(o.constant_values, dtype=np.float64)
        self.constant_names = list(o.constants)
        self.base_dir = base_dir
        self._build_guess()

    @classmethod
    def from_file(cls, path):
        import os
        with open(path) as f:
            return cls(f.read(), name=os.path.splitext(os.path.basename(path))[0],
                       base_dir=os.path.dirname(os.path.abspath(path)))

    # -- initial guess, as the generated BvpDae.__init__ builds it --
    def _estimate_fn(self, exprs):
        """Evaluate estimate expressions the way the generated module does:
        str(sympy expr) evaluated with `t` and the constants bound and math's
        names in scope."""
        if not exprs:
            return None
        code = [compile(str(e), "<estimate>", "eval") for e in exprs]
        base = {k: getattr(math, k) for k in dir(math) if not k.startswith("_")}
        for name, v in zip(self.spec.constants, self.spec.constant_values):
            base[name] = v

        def fn(t):
            env = dict(base)
            env["t"] = t
            return [eval(c, {"__builtins__": {}}, env) for c in code]
        return fn

    def _apply_estimates(self, T, Y, Z, P):
        o = self.spec
        if not (o.state_estimate or o.control_estimate or o.parameter_estimate):
            return
        se, ce = self._estimate_fn(o.state_estimate), self._estimate_fn(o.control_estimate)
        for i in range(T.shape[0]):
            t = float(T[i])
            if se:
                for j, v in enumerate(se(t)):
                    Y[i][j] = v
            if ce:
                for j, v in enumerate(ce(t)):
                    Z[i][j] = v
        if P.shape[0] != 0 and o.parameter_estimate:
            pe = self._estimate_fn(o.parameter_estimate)(0.0)
            for j, v in enumerate(pe):
                P[j] = v

    def _default_guess(self):
        o = self.spec
        N = o.nodes
        T0 = np.linspace(o.t_i, o.t_f, N)
        Y0 = np.ones((N, self.size_y), dtype=np.float64)
        Z0 = np.ones((N, self.size_z), dtype=np.float64)
        P0 = np.ones(self.size_p, dtype=np.float64) if self.size_p > 0 else np.ones(0, dtype=np.float64)
        return N, T0, Y0, Z0, P0

    def _build_guess(self):
        from .io import bvpdae_read_data
        o = self.spec
        if o.input_file:
            import os
            path = o.input_file
            if self.base_dir and not os.path.isabs(path) and not os.path.exists(path):
                path = os.path.join(self.base_dir, path)
            error, t0, y0, z0, p0 = bvpdae_read_data(path)
            if error != 0:
                print("Unable to read input file!")
                N, T0, Y0, Z0, P0 = self._default_guess()
                self._apply_estimates(T0, Y0, Z0, P0)
            else:
                print("Read input file!")
                N = t0.shape[0]
                T0 = t0
                Y0 = np.ones((N, self.size_y), dtype=np.float64) if self.size_y > 0 else None
                Z0 = np.ones((N, self.size_z), dtype=np.float64) if self.size_z > 0 else None
                P0 = np.ones(self.size_p, dtype=np.float64) if self.size_p > 0 else None
                if Y0 is not None and y0 is not None:
                    mm = min(y0.shape[1], Y0.shape[1])
                    Y0[:N, :mm] = y0[:N, :mm]
                if Z0 is not None and z0 is not None:
                    mm = min(z0.shape[1], len(o.u))
                    Z0[:N, :mm] = z0[:N, :mm]
                if P0 is not None and p0 is not None:
                    mm = min(p0.shape[0], P0.shape[0])
                    P0[:mm] = p0[:mm]
                self._apply_estimates(T0, Y0, Z0, P0)
        else:
            N, T0, Y0, Z0, P0 = self._default_guess()
            self._apply_estimates(T0, Y0, Z0, P0)
        self.N, self.T0, self.Y0, self.Z0, self.P0 = N, T0, Y0, Z0, P0
        self.t_initial, self.t_final = o.t_i, o.t_f


def problem_from_text(text, name="ocp"):
    return Problem(text, name=name)


def problem_from_file(path):
    return Problem.from_file(path)
