"""Python objects over the C ABI: a compiled problem (one m) and a batch of
instances in HBM.

    prob = Problem.from_file("vdp.ocp")
    cp = CompiledProblem(prob, m=4)            # NVRTC, cached
    bt = Batch(cp, n_instances)
    bt.set_guess([(t, y, z), ...], p, theta)   # host arrays, packed on device
    bt.solve(opts)
    sols = bt.solution()                       # list of dicts (t, y, z, p, stats)
"""
import ctypes
import os
import sys

import numpy as np

from . import _lib
from .codegen import ProblemCode, cuda_problem_source
from .tables import lobatto, segment_tables

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_CACHE = os.path.join(HERE, "_build", "nvrtc_cache")


def _tables(m):
    rk = lobatto(m)
    st = segment_tables(m)
    arr = lambda a: np.ascontiguousarray(a, dtype=np.float64).ravel()  # noqa: E731
    return dict(A=arr(rk.A), b=arr(rk.b), c=arr(rk.c), gw=arr(st["w"]), gL=arr(st["L"]), gI=arr(st["I"]),
                L0=arr(st["L0"]), L1=arr(st["L1"]))


def kernel_program_text(problem, m, big=False, smem_max=232448):
    """The NVRTC program for (problem, m) as one CUDA source (used for nvcc
    compile checks; the library builds the same text at run time).  big:
    the large-system kernels (condensation and tree)."""
    pc = ProblemCode(problem.sym)
    t = _tables(m)

    def arr(name, a):
        return "__constant__ double %s[%d] = {%s};\n" % (name, a.size, ",".join("%.17e" % v for v in a) or "0.0")

    out = "#define CS_NY %d\n#define CS_NZ %d\n#define CS_NP %d\n#define CS_NPE %d\n#define CS_NTH %d\n#define CS_M %d\n" % (
        pc.ny, pc.nz, pc.np, pc.np_eff, pc.nth, m)
    if big:
        out += "#define CS_BIG_COND 1\n#define CS_BIG_TREE 1\n#define CS_SMEM_MAX %d\n" % smem_max
    out += arr("CS_A", t["A"]) + arr("CS_B", t["b"]) + arr("CS_C", t["c"]) + arr("CS_GW", t["gw"])
    out += arr("CS_GL", t["gL"]) + arr("CS_GI", t["gI"]) + arr("CS_L0", t["L0"]) + arr("CS_L1", t["L1"])
    out += cuda_problem_source(pc)
    out += open(os.path.join(HERE, "csrc", "cs_umma.cuh")).read() + "\n"
    out += open(os.path.join(HERE, "csrc", "cs_kernels.cuh")).read()
    return out


class CompiledProblem:
    """A problem compiled for the GPU with m collocation points.

    layout: 0 automatic, 1 shared-memory kernels only, 2 the large-system
    kernels (global-memory slab per CTA; chosen automatically when a stage
    system or a BABD block does not fit in shared memory).
    precision: "fp64" (default), "tf32" or "bf16": the large-system
    condensation on the tensor cores (an inexact Newton Jacobian; residual,
    line search, mesh error and BABD solve stay FP64); "tf32-tree" /
    "bf16-tree" also run the tree merges' block updates on them."""

    PRECISIONS = {"fp64": 0, "tf32": 1, "bf16": 2, "tf32-tree": 3, "bf16-tree": 4}

    def __init__(self, problem, m, cache_dir=DEFAULT_CACHE, layout=0, precision="fp64"):
        lib = _lib.load()
        self.problem = problem
        self.m = m
        generated = isinstance(problem, GeneratedProblem)
        pc = problem.code if generated else ProblemCode(problem.sym)
        self.pc = pc
        self.ny, self.nz, self.np, self.np_eff, self.nth = pc.ny, pc.nz, pc.np, pc.np_eff, pc.nth
        self.s = m * (pc.ny + pc.nz)
        self.rowsz = pc.ny * (2 * pc.ny + pc.np_eff + 1)
        self._src = (problem.cuda_source if generated else cuda_problem_source(pc)).encode()
        self._t = _tables(m)
        self._cache = (cache_dir or "").encode()
        d = _lib.ModuleDesc()
        d.problem_src = self._src
        d.ny, d.nz, d.np, d.np_eff, d.n_theta, d.m = pc.ny, pc.nz, pc.np, pc.np_eff, pc.nth, m
        d.lobatto_A, d.lobatto_b, d.lobatto_c = (_lib.dptr(self._t[k]) for k in ("A", "b", "c"))
        d.gauss_w, d.gauss_L, d.gauss_I = (_lib.dptr(self._t[k]) for k in ("gw", "gL", "gI"))
        d.L0, d.L1 = _lib.dptr(self._t["L0"]), _lib.dptr(self._t["L1"])
        d.cache_dir = self._cache if cache_dir else None
        d.layout = int(layout)
        self.layout = int(layout)
        d.precision = self.PRECISIONS[precision]
        self.precision = precision
        h = ctypes.c_void_p()
        _lib.check(lib.cs_module_load(ctypes.byref(d), ctypes.byref(h)), "cs_module_load")
        self.handle = h
        self._lib = lib

    def __del__(self):
        if sys.is_finalizing():  # the CUDA runtime may already be gone
            return
        try:
            if getattr(self, "handle", None):
                self._lib.cs_module_free(self.handle)
                self.handle = None
        except Exception:  # noqa: BLE001
            pass


class GeneratedProblem:
    """A problem given by its generated CUDA problem functions (the text
    codegen.cuda_problem_source emits) with its sizes, constants and solver
    settings, without the OCP front end and sympy: for machines that only
    solve problems prepared elsewhere (from_problem makes one from a
    front-end Problem; the fields can be stored and loaded as plain arrays)."""

    def __init__(self, cuda_source, ny, nz, np_, np_eff, nth, theta=(), tolerance=1e-6,
                 maximum_newton_iterations=200, maximum_mesh_refinements=10, maximum_nodes=2000, size_inequality=0,
                 size_sv_inequality=0, name="generated"):
        import types
        self.cuda_source = str(cuda_source)
        self.code = types.SimpleNamespace(ny=int(ny), nz=int(nz), np=int(np_), np_eff=int(np_eff), nth=int(nth))
        self.size_y, self.size_z, self.size_p = int(ny), int(nz), int(np_)
        self.theta = np.asarray(theta, dtype=np.float64).reshape(-1)
        self.tolerance = float(tolerance)
        self.maximum_newton_iterations = int(maximum_newton_iterations)
        self.maximum_mesh_refinements = int(maximum_mesh_refinements)
        self.maximum_nodes = int(maximum_nodes)
        self.size_inequality = int(size_inequality)
        self.size_sv_inequality = int(size_sv_inequality)
        self.name = name

    @classmethod
    def from_problem(cls, pr, name="generated"):
        pc = ProblemCode(pr.sym)
        return cls(cuda_problem_source(pc), pc.ny, pc.nz, pc.np, pc.np_eff, pc.nth, pr.theta, pr.tolerance,
                   pr.maximum_newton_iterations, pr.maximum_mesh_refinements, pr.maximum_nodes, pr.size_inequality,
                   pr.size_sv_inequality, name=name)

    @classmethod
    def from_arrays(cls, d):
        """From a mapping of plain values (e.g. an npz file's arrays)."""
        return cls(str(d["cuda_source"]), int(d["ny"]), int(d["nz"]), int(d["np"]), int(d["np_eff"]), int(d["nth"]),
                   d["theta"], float(d["tolerance"]), int(d["maximum_newton_iterations"]),
                   int(d["maximum_mesh_refinements"]), int(d["maximum_nodes"]), int(d["size_inequality"]),
                   int(d["size_sv_inequality"]), name=str(d.get("name", "generated")))


def default_opts(problem=None, **kw):
    """cs_opts from the problem's BvpDae attributes and the reference's
    constants (alpha0 0.1, beta 0.9, alpha_m 1e-6 with inequalities else 0.1)."""
    lib = _lib.load()
    o = _lib.Opts()
    lib.cs_opts_default(ctypes.byref(o))
    if problem is not None:
        o.tol = problem.tolerance
        o.max_iter = problem.maximum_newton_iterations
        o.max_mesh = problem.maximum_mesh_refinements
        o.max_nodes = problem.maximum_nodes
        o.alpha_m = 1e-6 if (problem.size_inequality > 0 or problem.size_sv_inequality > 0) else 0.1
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Batch:
    """A batch of instances of one compiled problem, resident in HBM."""

    def __init__(self, cp, n_instances, node_capacity=0, stream=None):
        self.cp = cp
        self.B = int(n_instances)
        lib = cp._lib
        h = ctypes.c_void_p()
        _lib.check(lib.cs_batch_create(cp.handle, self.B, int(node_capacity), stream, ctypes.byref(h)), "cs_batch_create")
        self.handle = h
        self._lib = lib

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            if getattr(self, "handle", None):
                self._lib.cs_batch_free(self.handle)
                self.handle = None
        except Exception:  # noqa: BLE001
            pass

    # ---- data in
    def set_guess_packed(self, N, t, y, z, p, theta=None):
        cp = self.cp
        N = np.ascontiguousarray(N, dtype=np.int32)
        t = np.ascontiguousarray(t, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64) if cp.nz > 0 else None
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(self.B, cp.np) if cp.np > 0 else None
        th = None
        if cp.nth > 0:
            th = np.ascontiguousarray(theta if theta is not None else np.tile(cp.problem.theta, (self.B, 1)),
                                      dtype=np.float64).reshape(self.B, cp.nth)
        assert N.shape == (self.B,)
        T = int(N.sum())
        assert t.shape == (T,) and y.shape == (T, cp.ny)
        if z is not None:
            assert z.shape == (T, cp.nz)
        _lib.check(self._lib.cs_batch_set_guess(self.handle, _lib.iptr(N), _lib.dptr(t), _lib.dptr(y), _lib.dptr(z),
                                                _lib.dptr(p), _lib.dptr(th)), "cs_batch_set_guess")

    def set_guess(self, meshes, p, theta=None):
        """meshes: list of (t, y, z) per instance (z may be None if nz == 0)."""
        N = np.array([len(m[0]) for m in meshes], dtype=np.int32)
        t = np.concatenate([np.asarray(m[0], dtype=np.float64) for m in meshes])
        y = np.concatenate([np.asarray(m[1], dtype=np.float64).reshape(-1, self.cp.ny) for m in meshes])
        z = np.concatenate([np.asarray(m[2], dtype=np.float64).reshape(-1, self.cp.nz) for m in meshes]) \
            if self.cp.nz > 0 else None
        self.set_guess_packed(N, t, y, z, p, theta)

    def set_state(self, meshes, p, theta=None):
        """meshes: list of (t, y, y_dot, z_tilde) per instance with the
        reference's shapes: y (N, ny), y_dot ((N-1) m, ny), z_tilde ((N-1) m, nz)."""
        cp = self.cp
        N = np.array([len(m[0]) for m in meshes], dtype=np.int32)
        t = np.ascontiguousarray(np.concatenate([np.asarray(m[0], float) for m in meshes]))
        y = np.ascontiguousarray(np.concatenate([np.asarray(m[1], float).reshape(-1, cp.ny) for m in meshes]))
        yd = np.ascontiguousarray(np.concatenate([np.asarray(m[2], float).reshape(-1, cp.m * cp.ny) for m in meshes]))
        zt = np.ascontiguousarray(np.concatenate([np.asarray(m[3], float).reshape(-1, cp.m * cp.nz) for m in meshes])) \
            if cp.nz > 0 else None
        p = np.ascontiguousarray(np.asarray(p, float).reshape(self.B, cp.np)) if cp.np > 0 else None
        th = None
        if cp.nth > 0:
            th = np.ascontiguousarray(theta if theta is not None else np.tile(cp.problem.theta, (self.B, 1)),
                                      dtype=np.float64).reshape(self.B, cp.nth)
        _lib.check(self._lib.cs_batch_set_state(self.handle, _lib.iptr(N), _lib.dptr(t), _lib.dptr(y), _lib.dptr(yd),
                                                _lib.dptr(zt), _lib.dptr(p), _lib.dptr(th)), "cs_batch_set_state")

    def reset(self):
        """Back to the last initial guess (device copy, no host transfer)."""
        _lib.check(self._lib.cs_batch_reset(self.handle), "cs_batch_reset")

    def profile_reset(self, timing=False):
        _lib.check(self._lib.cs_profile_reset(self.handle, int(bool(timing))), "cs_profile_reset")

    def profile(self):
        pr = _lib.Profile()
        _lib.check(self._lib.cs_profile_get(self.handle, ctypes.byref(pr)), "cs_profile_get")
        return {k: getattr(pr, k) for k, _ in _lib.Profile._fields_}

    # ---- solve
    def solve(self, opts=None):
        o = opts if opts is not None else default_opts(self.cp.problem)
        _lib.check(self._lib.cs_solve(self.handle, ctypes.byref(o)), "cs_solve")

    def set_progress(self, fn):
        """fn(active, super_steps) is called on the solving thread after each
        check of the Newton phase (instances still iterating, super-steps so
        far); the batch may be read from it (statuses()), not solved.  None
        removes it."""
        if fn is None:
            self._progress = None
            cb = ctypes.cast(None, _lib.PROGRESS_FN)
        else:
            def tramp(_user, active, steps):
                fn(int(active), int(steps))
            cb = _lib.PROGRESS_FN(tramp)
            self._progress = cb  # keeps the ctypes thunk alive
        _lib.check(self._lib.cs_batch_set_progress(self.handle, cb, None), "cs_batch_set_progress")

    def statuses(self):
        """Per-instance status codes (0 fresh, 1 line search, 2 segment
        residual, 3 done, 4 failed, 5 remesh, 6 parked spare, 7 stopped
        spare) without copying the solution."""
        st = (_lib.Stats * self.B)()
        _lib.check(self._lib.cs_get_solution(self.handle, None, None, None, None, st), "cs_get_solution")
        return np.ctypeslib.as_array(st)["status"].astype(np.int32)

    # ---- data out
    def sizes(self):
        N = np.zeros(self.B, dtype=np.int32)
        T = ctypes.c_longlong()
        _lib.check(self._lib.cs_batch_sizes(self.handle, _lib.iptr(N), ctypes.byref(T)), "cs_batch_sizes")
        return N, int(T.value)

    def solution_packed(self):
        cp = self.cp
        N, T = self.sizes()
        t = np.zeros(T)
        y = np.zeros((T, cp.ny))
        z = np.zeros((T, max(cp.nz, 1)))
        p = np.zeros((self.B, max(cp.np, 1)))
        st = (_lib.Stats * self.B)()
        _lib.check(self._lib.cs_get_solution(self.handle, _lib.dptr(t), _lib.dptr(y), _lib.dptr(z), _lib.dptr(p), st),
                   "cs_get_solution")
        return N, t, y, z[:, :cp.nz], p[:, :cp.np], st

    def solution(self, indices=None, packed=None):
        """Per-instance solution dicts, of every instance or of `indices`
        (from `packed`, a solution_packed() result, if given)."""
        N, t, y, z, p, st = self.solution_packed() if packed is None else packed
        off = np.concatenate(([0], np.cumsum(N, dtype=np.int64)))
        out = []
        for b in (range(self.B) if indices is None else indices):
            o, n = int(off[b]), int(N[b])
            s = st[b]
            out.append(dict(N=n, t=t[o:o + n], y=y[o:o + n], z=z[o:o + n], p=p[b],
                            status=int(s.status), success=int(s.status) == 3, newton_steps=int(s.newton_steps),
                            residual_evals=int(s.residual_evals), segment_evals=int(s.segment_evals),
                            remeshes=int(s.remeshes), continuation_steps=int(s.continuation_steps),
                            alpha=float(s.alpha), max_residual=float(s.max_residual), last_norm=float(s.last_norm),
                            singular=int(s.singular), fail_reason=int(s.fail_reason)))
        return out

    def solution_text(self):
        """Every instance's solution file (the reference's text format, the
        numbers as "{}".format prints them), formatted on the GPU: the text of
        all files (a memoryview of bytes, not copied again) and their byte
        offsets (file b is text[off[b]:off[b + 1]])."""
        off = np.zeros(self.B + 1, dtype=np.int64)
        _lib.check(self._lib.cs_format_solutions(self.handle, None, 0, off.ctypes.data), "cs_format_solutions")
        buf = np.empty(max(int(off[-1]), 1), dtype=np.uint8)
        _lib.check(self._lib.cs_format_solutions(self.handle, buf.ctypes.data, int(off[-1]), off.ctypes.data),
                   "cs_format_solutions")
        return memoryview(buf)[:int(off[-1])], off

    def state(self):
        cp = self.cp
        N, T = self.sizes()
        t = np.zeros(T)
        y = np.zeros((T, cp.ny))
        yd = np.zeros((T, cp.m, cp.ny))
        zt = np.zeros((T, cp.m, max(cp.nz, 1)))
        zn = np.zeros((T, max(cp.nz, 1)))
        p = np.zeros((self.B, max(cp.np, 1)))
        _lib.check(self._lib.cs_get_state(self.handle, _lib.dptr(t), _lib.dptr(y), _lib.dptr(yd), _lib.dptr(zt),
                                          _lib.dptr(zn), _lib.dptr(p)), "cs_get_state")
        return dict(N=N, t=t, y=y, ydot=yd, zt=zt[:, :, :cp.nz], z=zn[:, :cp.nz], p=p[:, :cp.np])

    # ---- stages
    def stage_residual(self, alpha, pieces=False):
        cp = self.cp
        _, T = self.sizes()
        norms = np.zeros(self.B)
        fa = np.zeros((T, cp.s)) if pieces else None
        fb = np.zeros((T, cp.ny)) if pieces else None
        _lib.check(self._lib.cs_stage_residual(self.handle, alpha, _lib.dptr(norms), _lib.dptr(fa), _lib.dptr(fb)),
                   "cs_stage_residual")
        return norms, fa, fb

    def stage_newton_direction(self, alpha):
        cp = self.cp
        _, T = self.sizes()
        rows = np.zeros((T, cp.rowsz))
        dy = np.zeros((T, cp.ny))
        dyd = np.zeros((T, cp.m, cp.ny))
        dzt = np.zeros((T, cp.m, max(cp.nz, 1)))
        dp = np.zeros((self.B, max(cp.np, 1)))
        _lib.check(self._lib.cs_stage_newton_direction(self.handle, alpha, _lib.dptr(rows), _lib.dptr(dy),
                                                       _lib.dptr(dyd), _lib.dptr(dzt), _lib.dptr(dp)),
                   "cs_stage_newton_direction")
        return dict(rows=rows, dy=dy, dydot=dyd, dzt=dzt[:, :, :cp.nz], dp=dp[:, :cp.np])

    def set_opts(self, opts):
        """Options of the stage entry points (segment residual estimate)."""
        _lib.check(self._lib.cs_batch_set_opts(self.handle, ctypes.byref(opts)), "cs_batch_set_opts")

    def stage_segment_residual(self, alpha, tol):
        _, T = self.sizes()
        res = np.zeros(T)
        mx = np.zeros(self.B)
        _lib.check(self._lib.cs_stage_segment_residual(self.handle, alpha, tol, _lib.dptr(res), _lib.dptr(mx)),
                   "cs_stage_segment_residual")
        return res, mx

    def stage_remesh(self, res):
        res = np.ascontiguousarray(res, dtype=np.float64)
        N = np.zeros(self.B, dtype=np.int32)
        _lib.check(self._lib.cs_stage_remesh(self.handle, _lib.dptr(res), _lib.iptr(N)), "cs_stage_remesh")
        return N

    def warm_start(self, traj_dev, n_nodes, stride):
        """Initial guess from per-instance trajectory vectors in device memory
        (row b of `traj_dev`, a DeviceArray or device address)."""
        ptr = traj_dev.ptr if isinstance(traj_dev, DeviceArray) else traj_dev
        _lib.check(self._lib.cs_batch_warm_start(self.handle, int(n_nodes), ctypes.c_void_p(ptr), int(stride)),
                   "cs_batch_warm_start")

    def set_spares(self, n_primary, trigger):
        """Pair instance k < n_primary (the primary) with instance
        n_primary + k (its spare: the same instance from another guess) on a
        batch of 2 n_primary instances.  Spares stay parked until at most
        `trigger` instances are in Newton (never if trigger < 0); from then on
        the spare of every primary still iterating or failed runs in the same
        super-steps, and every failed primary's spare has run when solve()
        returns.  warm_start() then fills only the primaries.  n_primary = 0
        removes the pairing."""
        _lib.check(self._lib.cs_batch_set_spares(self.handle, int(n_primary), int(trigger)), "cs_batch_set_spares")

    def autotune(self, reps=3):
        """Time the condensation's launch shapes on this batch's intervals and
        keep the fastest for the compiled problem (all its batches)."""
        r = _lib.TuneResult()
        _lib.check(self._lib.cs_autotune_condense(self.handle, int(reps), ctypes.byref(r)), "cs_autotune_condense")
        return dict(lanes=r.lanes, block=r.block, grid=r.grid, candidates=r.candidates, ms=r.ms,
                    default_ms=r.default_ms)

    def time_condense(self, reps=10):
        ms = ctypes.c_double()
        _lib.check(self._lib.cs_time_condense(self.handle, int(reps), ctypes.byref(ms)), "cs_time_condense")
        return ms.value


class DeviceArray:
    """Device memory of a given shape/dtype with host copies in and out."""

    def __init__(self, shape, dtype=np.float32):
        lib = _lib.load()
        self._lib = lib
        self.shape = tuple(shape)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self.ptr = lib.cs_device_alloc(max(self.nbytes, 8))
        if not self.ptr:
            raise _lib.CsError("device allocation failed: " + _lib.last_error())

    def upload(self, a):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.nbytes <= self.nbytes
        _lib.check(self._lib.cs_copy(ctypes.c_void_p(self.ptr), a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 0), "cs_copy")

    def download(self):
        out = np.empty(self.shape, self.dtype)
        _lib.check(self._lib.cs_copy(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(self.ptr), self.nbytes, 1),
                   "cs_copy")
        return out

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            if self.ptr:
                self._lib.cs_device_free(ctypes.c_void_p(self.ptr))
                self.ptr = None
        except Exception:  # noqa: BLE001
            pass


class PinnedArray:
    """numpy array over page-locked host memory (freed with the object)."""

    def __init__(self, shape, dtype=np.float64):
        lib = _lib.load()
        self._lib = lib
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = lib.cs_pinned_alloc(max(n, 8))
        if not self.ptr:
            raise _lib.CsError("pinned allocation failed: " + _lib.last_error())
        buf = (ctypes.c_char * max(n, 8)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            if self.ptr:
                self._lib.cs_pinned_free(self.ptr)
                self.ptr = None
        except Exception:  # noqa: BLE001
            pass


def measure_fp64_peak():
    lib = _lib.load()
    v = ctypes.c_double()
    _lib.check(lib.cs_measure_fp64_peak(ctypes.byref(v)), "cs_measure_fp64_peak")
    return v.value


def measure_dmma_peak():
    """FP64 tensor-core (DMMA) throughput in TFLOP/s (register-resident loop)."""
    lib = _lib.load()
    v = ctypes.c_double()
    _lib.check(lib.cs_measure_dmma_peak(ctypes.byref(v)), "cs_measure_dmma_peak")
    return v.value
