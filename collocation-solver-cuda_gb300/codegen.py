"""Emit the problem functions of a derived BVP-DAE as code.

Two targets:

* CUDA C device functions, compiled with NVRTC together with the solver
  kernels (csrc/kernels.cuh).  The reference emits the same six functions as
  numba device functions via sympy.ccode (OCP2ABVP.py:184-327); the interface
  here keeps its argument meaning, with the instance constants `th` added:

      cs_f (y, z, p, th, f)            f  : [NY]
      cs_g (y, z, p, th, alpha, g)     g  : [NZ]
      cs_Df(y, z, p, th, Df)           Df : [NY][NY+NZ+NP], every entry written
      cs_Dg(y, z, p, th, alpha, Dg)    Dg : [NZ][NY+NZ+NP], every entry written
      cs_r (y0, y1, p, th, r)          r  : [NY+NP]
      cs_Dr(y0, y1, p, th, Dr)         Dr : [NY+NP][2NY+NP] (columns y0, y1, p)

  Common subexpressions are shared (sympy.cse), small integer powers become
  products and x**(1/2) becomes sqrt: GB300 has little FP64 throughput, and
  pow() would cost far more than the multiplications it stands for.
  Transcendentals call CUDA's own sin/cos/exp/... .

* numpy functions over arrays of points (one row per point), used by the host
  code and by tests; same six functions, vectorised.
"""
import keyword

import numpy as np
import sympy
from sympy.printing.c import C99CodePrinter
from sympy.printing.numpy import NumPyPrinter
from sympy.printing.precedence import precedence


class _CudaPrinter(C99CodePrinter):
    def _print_Float(self, expr):
        v = float(expr)
        s = repr(v)
        if "e" not in s and "." not in s and "inf" not in s and "nan" not in s:
            s += ".0"
        return s

    def _print_Integer(self, expr):
        return "%d.0" % int(expr)

    def _print_Rational(self, expr):
        return "(%s/%s)" % (self._print_Integer(sympy.Integer(expr.p)), self._print_Integer(sympy.Integer(expr.q)))

    def _print_Pow(self, expr):
        b, e = expr.base, expr.exp
        pb = self.parenthesize(b, precedence(expr))
        if e.is_Integer:
            n = int(e)
            if n == 1:
                return self._print(b)
            if 2 <= n <= 4:
                return "(" + "*".join([pb] * n) + ")"
            if -4 <= n <= -1:
                return "(1.0/(" + "*".join([pb] * (-n)) + "))"
        if e == sympy.S.Half:
            return "sqrt(%s)" % self._print(b)
        if e == -sympy.S.Half:
            return "(1.0/sqrt(%s))" % self._print(b)
        return "pow(%s, %s)" % (self._print(b), self._print(e))


class _NpPrinter(NumPyPrinter):
    def _print_Float(self, expr):
        return repr(float(expr))

    def _print_Rational(self, expr):
        return "(%r/%r)" % (float(expr.p), float(expr.q))


def _rename(sym_problem):
    """Map the problem's symbols to code-safe names: y -> cs_y<i>, etc."""
    s = sym_problem
    m = {}
    for i, v in enumerate(s.y):
        m[v] = sympy.Symbol("cs_y%d" % i)
    for i, v in enumerate(s.z):
        m[v] = sympy.Symbol("cs_z%d" % i)
    for i, v in enumerate(s.p):
        m[v] = sympy.Symbol("cs_p%d" % i)
    for i, v in enumerate(s.theta):
        m[v] = sympy.Symbol("cs_th%d" % i)
    m[s.alpha] = sympy.Symbol("cs_alpha")
    return m


def _cse(exprs, prefix):
    syms = sympy.numbered_symbols(prefix)
    reps, red = sympy.cse(exprs, symbols=syms, optimizations="basic")
    return reps, red


def _free(exprs):
    out = set()
    for e in exprs:
        out |= e.free_symbols
    return out


class ProblemCode:
    """Symbolic blocks of a problem, renamed and ready to print."""

    def __init__(self, sym_problem):
        s = sym_problem
        self.sym = s
        self.ny, self.nz, self.np = s.ny, s.nz, s.np
        self.nth = len(s.theta)
        self.np_eff = s.np_eff
        ren = _rename(s)
        self.ren = ren
        sub = lambda e: sympy.sympify(e).xreplace(ren)  # noqa: E731
        self.f = [sub(e) for e in s.f]
        self.g = [sub(e) for e in s.g]
        Df, Dg = s.jac_fg()
        self.Df = [[sub(e) for e in row] for row in Df]
        self.Dg = [[sub(e) for e in row] for row in Dg]
        y0, y1, r, Dr = s.bc_exprs()
        bren = dict(ren)
        for i in range(s.ny):
            bren[y0[i]] = sympy.Symbol("cs_a%d" % i)
            bren[y1[i]] = sympy.Symbol("cs_b%d" % i)
        self.r = [sympy.sympify(e).xreplace(bren) for e in r]
        self.Dr = [[sympy.sympify(e).xreplace(bren) for e in row] for row in Dr]
        self.Df_nz = np.array([[e != 0 for e in row] for row in self.Df], dtype=bool).reshape(self.ny, self.ny + self.nz + self.np)
        self.Dg_nz = np.array([[e != 0 for e in row] for row in self.Dg], dtype=bool).reshape(self.nz, self.ny + self.nz + self.np)


# ------------------------------------------------------------------ CUDA ---
def _cuda_prologue(used, kinds):
    lines = []
    for name in sorted(used, key=lambda v: v.name):
        n = name.name
        if n.startswith("cs_y") and "y" in kinds:
            lines.append("  const double %s = y[%s];" % (n, n[4:]))
        elif n.startswith("cs_z"):
            lines.append("  const double %s = z[%s];" % (n, n[4:]))
        elif n.startswith("cs_p"):
            lines.append("  const double %s = p[%s];" % (n, n[4:]))
        elif n.startswith("cs_th"):
            lines.append("  const double %s = th[%s];" % (n, n[5:]))
        elif n.startswith("cs_a"):
            lines.append("  const double %s = y0[%s];" % (n, n[4:]))
        elif n.startswith("cs_b"):
            lines.append("  const double %s = y1[%s];" % (n, n[4:]))
    return lines


def _cuda_body(exprs, targets, pr):
    reps, red = _cse(exprs, "cs_t")
    used = _free([e for _, e in reps] + red)
    lines = _cuda_prologue(used - {s for s, _ in reps} - {sympy.Symbol("cs_alpha")}, ("y",))
    for s_, e in reps:
        lines.append("  const double %s = %s;" % (s_.name, pr.doprint(e)))
    for tgt, e in zip(targets, red):
        lines.append("  %s = %s;" % (tgt, pr.doprint(e)))
    return lines


def _cuda_matrix(flat, name, pr):
    """Assignments of a flattened derivative matrix.  Large, mostly
    structurally zero matrices (pendulum chains: Df, Dr of thousands of
    entries, a few percent nonzero) are cleared by a loop and only their
    nonzeros assigned, which keeps the generated code, and its compile time,
    proportional to the nonzeros."""
    n = len(flat)
    nz = [k for k, e in enumerate(flat) if e != 0]
    if n > 256 and len(nz) < n // 2:
        lines = ["  for (int cs_k = 0; cs_k < %d; ++cs_k) %s[cs_k] = 0.0;" % (n, name)]
        if nz:
            lines += _cuda_body([flat[k] for k in nz], ["%s[%d]" % (name, k) for k in nz], pr)
        return lines
    return _cuda_body(flat, ["%s[%d]" % (name, k) for k in range(n)], pr) if flat else []


def cuda_problem_source(pc):
    """CUDA C text for the six problem functions of ProblemCode `pc`."""
    pr = _CudaPrinter()
    ny, nz, npar = pc.ny, pc.nz, pc.np
    nc = ny + nz + npar
    out = []
    sig_pt = "const double* __restrict__ y, const double* __restrict__ z, const double* __restrict__ p, const double* __restrict__ th"
    sig_bc = "const double* __restrict__ y0, const double* __restrict__ y1, const double* __restrict__ p, const double* __restrict__ th"
    A = "__device__ __forceinline__ void"

    out.append("%s cs_f(%s, double* __restrict__ f) {" % (A, sig_pt))
    out += _cuda_body(pc.f, ["f[%d]" % i for i in range(ny)], pr) if ny else []
    out.append("}")
    out.append("%s cs_g(%s, const double cs_alpha, double* __restrict__ g) {" % (A, sig_pt))
    out.append("  (void)cs_alpha;")
    out += _cuda_body(pc.g, ["g[%d]" % i for i in range(nz)], pr) if nz else []
    out.append("}")
    out.append("%s cs_Df(%s, double* __restrict__ Df) {" % (A, sig_pt))
    out += _cuda_matrix([e for row in pc.Df for e in row], "Df", pr)
    out.append("}")
    out.append("%s cs_Dg(%s, const double cs_alpha, double* __restrict__ Dg) {" % (A, sig_pt))
    out.append("  (void)cs_alpha;")
    out += _cuda_matrix([e for row in pc.Dg for e in row], "Dg", pr)
    out.append("}")
    out.append("%s cs_r(%s, double* __restrict__ r) {" % (A, sig_bc))
    out += _cuda_body(pc.r, ["r[%d]" % i for i in range(len(pc.r))], pr)
    out.append("}")
    out.append("%s cs_Dr(%s, double* __restrict__ Dr) {" % (A, sig_bc))
    out += _cuda_matrix([e for row in pc.Dr for e in row], "Dr", pr)
    out.append("}")
    return "\n".join(out) + "\n"


# ----------------------------------------------------------------- numpy ---
def _np_body(exprs, name_fmt, npr):
    reps, red = _cse(exprs, "cs_t")
    lines = []
    for s_, e in reps:
        lines.append("    %s = %s" % (s_.name, npr.doprint(e)))
    for k, e in enumerate(red):
        lines.append("    " + name_fmt % k + " = " + npr.doprint(e))
    return lines


def numpy_problem_source(pc):
    """Python source defining vectorised f, g, Df, Dg, r, Dr.

    Point arrays have one row per point: y (n, ny), z (n, nz); p (np,) and
    th (nth,) are shared by all points; alpha is a float.  r and Dr take the
    node vectors y0, y1 (ny,).
    """
    npr = _NpPrinter({"fully_qualified_modules": True, "inline": True})
    ny, nz, npar = pc.ny, pc.nz, pc.np
    nc = ny + nz + npar
    L = ["import numpy", ""]

    def pro(kind):
        out = []
        if kind == "pt":
            out += ["    cs_y%d = y[:, %d]" % (i, i) for i in range(ny)]
            out += ["    cs_z%d = z[:, %d]" % (i, i) for i in range(nz)]
        else:
            out += ["    cs_a%d = y0[%d]" % (i, i) for i in range(ny)]
            out += ["    cs_b%d = y1[%d]" % (i, i) for i in range(ny)]
        out += ["    cs_p%d = p[%d]" % (i, i) for i in range(npar)]
        out += ["    cs_th%d = th[%d]" % (i, i) for i in range(pc.nth)]
        return out

    L += ["def f(y, z, p, th):", "    n = y.shape[0]"] + pro("pt") + ["    out = numpy.zeros((n, %d))" % ny]
    L += _np_body(pc.f, "out[:, %d]", npr) + ["    return out", ""]
    L += ["def g(y, z, p, th, cs_alpha):", "    n = y.shape[0]"] + pro("pt") + ["    out = numpy.zeros((n, %d))" % nz]
    L += (_np_body(pc.g, "out[:, %d]", npr) if nz else []) + ["    return out", ""]
    L += ["def Df(y, z, p, th):", "    n = y.shape[0]"] + pro("pt") + ["    out = numpy.zeros((n, %d))" % (ny * nc)]
    L += _np_body([e for row in pc.Df for e in row], "out[:, %d]", npr) + ["    return out.reshape(n, %d, %d)" % (ny, nc), ""]
    L += ["def Dg(y, z, p, th, cs_alpha):", "    n = y.shape[0]"] + pro("pt") + ["    out = numpy.zeros((n, %d))" % (nz * nc)]
    L += (_np_body([e for row in pc.Dg for e in row], "out[:, %d]", npr) if nz else []) + \
        ["    return out.reshape(n, %d, %d)" % (nz, nc), ""]
    L += ["def r(y0, y1, p, th):"] + pro("bc") + ["    out = numpy.zeros(%d)" % (ny + npar)]
    L += _np_body(pc.r, "out[%d]", npr) + ["    return out", ""]
    L += ["def Dr(y0, y1, p, th):"] + pro("bc") + ["    out = numpy.zeros(%d)" % ((ny + npar) * (2 * ny + npar))]
    L += _np_body([e for row in pc.Dr for e in row], "out[%d]", npr) + \
        ["    return out.reshape(%d, %d)" % (ny + npar, 2 * ny + npar), ""]
    return "\n".join(L)


class NumpyProblem:
    """Vectorised problem functions compiled from numpy_problem_source."""

    def __init__(self, pc):
        src = numpy_problem_source(pc)
        ns = {}
        exec(compile(src, "<problem:%s>" % id(pc), "exec"), ns)
        self.source = src
        self.f, self.g, self.Df, self.Dg, self.r, self.Dr = (ns[k] for k in ("f", "g", "Df", "Dg", "r", "Dr"))
        self.ny, self.nz, self.np, self.nth, self.np_eff = pc.ny, pc.nz, pc.np, pc.nth, pc.np_eff


def _check_ident(name):
    return name.isidentifier() and not keyword.iskeyword(name)
