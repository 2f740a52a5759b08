"""Learned warm start: an MLP maps the parameters of an OCP instance to its
state/costate/control trajectory at fixed normalised-time nodes; the
prediction, interpolated onto the instance's mesh, is the Newton initial
guess.  The network is trained and run by the library's own kernels
(csrc/cs_mlp.cu) on solutions the batched solver produces.

A warm-started solve is accepted only when it meets the tolerance; any
instance whose warm-started Newton iteration fails is solved again from the
plain initial guess (fallback).
"""
import collections
import ctypes
import sys
import threading

import numpy as np

from . import _lib
from .module import Batch, CompiledProblem, default_opts

N_NODES = 64


class Mlp:
    """The network (ctypes over cs_mlp_*)."""

    def __init__(self, n_in, n_out, width=256, depth=4, seed=0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.cs_mlp_create(n_in, width, depth, n_out, seed, ctypes.byref(h)), "cs_mlp_create")
        self.handle = h
        self.n_in, self.n_out, self.width, self.depth = n_in, n_out, width, depth
        self.sizes = [(n_in if l == 0 else width, n_out if l == depth - 1 else width) for l in range(depth)]
        self.norm = (np.zeros(n_in, np.float32), np.ones(n_in, np.float32), np.zeros(n_out, np.float32),
                     np.ones(n_out, np.float32))

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            if getattr(self, "handle", None):
                self._lib.cs_mlp_free(self.handle)
                self.handle = None
        except Exception:  # noqa: BLE001
            pass

    @property
    def n_params(self):
        return int(self._lib.cs_mlp_num_params(self.handle))

    def set_normalization(self, xm, xs, ym, ys):
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (xm, xs, ym, ys)]
        _lib.check(self._lib.cs_mlp_set_normalization(self.handle, *[_lib.fptr(a) for a in arrs]),
                   "cs_mlp_set_normalization")
        self.norm = tuple(arrs)

    def fit_normalization(self, X, Y):
        xs = X.std(axis=0)
        ys = Y.std(axis=0)
        self.set_normalization(X.mean(axis=0), np.where(xs > 1e-8, xs, 1.0), Y.mean(axis=0),
                               np.where(ys > 1e-8, ys, 1.0))

    def params(self):
        out = np.zeros(self.n_params, np.float32)
        _lib.check(self._lib.cs_mlp_get_params(self.handle, _lib.fptr(out)), "cs_mlp_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        _lib.check(self._lib.cs_mlp_set_params(self.handle, _lib.fptr(p)), "cs_mlp_set_params")

    def gradient(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        loss = ctypes.c_double()
        g = np.zeros(self.n_params, np.float32)
        _lib.check(self._lib.cs_mlp_gradient(self.handle, _lib.fptr(X), _lib.fptr(Y), X.shape[0], ctypes.byref(loss),
                                             _lib.fptr(g)), "cs_mlp_gradient")
        return loss.value, g

    def train(self, X, Y, epochs=200, batch=512, lr=1e-3, seed=0, lr_final=None):
        """Adam on mini-batches; lr_final (a fraction of lr): the rate decays
        along a half cosine to lr_final * lr over the run, else constant."""
        _lib.check(self._lib.cs_mlp_set_schedule(self.handle, ctypes.c_float(-1.0 if lr_final is None else lr_final)),
                   "cs_mlp_set_schedule")
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        loss = ctypes.c_double()
        _lib.check(self._lib.cs_mlp_train(self.handle, _lib.fptr(X), _lib.fptr(Y), X.shape[0], epochs, batch,
                                          ctypes.c_float(lr), seed, ctypes.byref(loss)), "cs_mlp_train")
        return loss.value

    def predict_device(self, dX, n, dY, stream=None):
        """Forward pass on device arrays (module.DeviceArray or addresses)."""
        px = dX.ptr if hasattr(dX, "ptr") else dX
        py = dY.ptr if hasattr(dY, "ptr") else dY
        _lib.check(self._lib.cs_mlp_predict_device(self.handle, ctypes.c_void_p(px), int(n), ctypes.c_void_p(py), stream),
                   "cs_mlp_predict_device")

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.n_out), np.float32)
        _lib.check(self._lib.cs_mlp_predict(self.handle, _lib.fptr(X), X.shape[0], _lib.fptr(Y)), "cs_mlp_predict")
        return Y


# ------------------------------------------------------- trajectories ---
def trajectory_vector(t, y, z, p, T, n_nodes=N_NODES):
    """y and z resampled at n_nodes equispaced normalised times in [0, 1]
    (linear interpolation of the nodal solution), then p."""
    s = np.linspace(0.0, 1.0, n_nodes)
    tau = t / T
    ys = np.stack([np.interp(s, tau, y[:, k]) for k in range(y.shape[1])], axis=1)
    zs = np.stack([np.interp(s, tau, z[:, k]) for k in range(z.shape[1])], axis=1) if z.shape[1] else np.zeros((n_nodes, 0))
    return np.concatenate([ys.ravel(), zs.ravel(), np.asarray(p, float).ravel()])


def guess_from_vector(v, t, T, ny, nz, npar, n_nodes=N_NODES):
    """Initial guess on the mesh t from a trajectory vector."""
    s = np.linspace(0.0, 1.0, n_nodes)
    ys = v[:n_nodes * ny].reshape(n_nodes, ny)
    zs = v[n_nodes * ny:n_nodes * (ny + nz)].reshape(n_nodes, nz)
    p = v[n_nodes * (ny + nz):n_nodes * (ny + nz) + npar]
    tau = t / T
    y = np.stack([np.interp(tau, s, ys[:, k]) for k in range(ny)], axis=1)
    z = np.stack([np.interp(tau, s, zs[:, k]) for k in range(nz)], axis=1) if nz else np.zeros((len(t), 0))
    return y, z, p


class Family:
    """An instance family: the OCP problem, instance parameters -> features,
    constants theta, final time, mesh and plain guess."""

    def __init__(self, problem, features, theta, final_time, plain_guess, name="family"):
        self.problem = problem
        self.features = features
        self.theta = theta
        self.final_time = final_time
        self.plain_guess = plain_guess
        self.name = name
        self.ny, self.nz, self.np = problem.size_y, problem.size_z, problem.size_p
        self.n_out = N_NODES * (self.ny + self.nz) + self.np


def vdp_family():
    from .workloads import vdp_family_problem
    pr = vdp_family_problem()
    return Family(pr, features=lambda i: np.array([i.x0[0], i.x0[1], i.T, np.log(i.r)]),
                  theta=lambda i: i.theta, final_time=lambda i: i.T, plain_guess=lambda i: i.guess(), name="vdp")


def pendulum_family(K=8):
    """Pendulum chain of K: features theta(0), T, k."""
    from .workloads import pendulum_family_problem
    pr = pendulum_family_problem(K)
    ny, nz, npar = pr.size_y, pr.size_z, pr.size_p
    return Family(pr, features=lambda i: np.concatenate([i.theta0, [i.T, i.k]]), theta=lambda i: i.theta,
                  final_time=lambda i: i.T, plain_guess=lambda i: i.guess(ny, nz, npar), name="pendulum%d" % K)


def write_guess_file(family, mlp, instance, path, n_nodes=None):
    """The network's trajectory for one instance, on its plain mesh (or
    n_nodes equispaced nodes), as a BVPDAEReadWriteData file: an OCP names it
    as InputFile to start from the learned guess.  Returns the status of the
    writer (0 on success)."""
    from .io import bvpdae_write_data
    X = np.array([family.features(instance)], np.float32)
    v = mlp.predict(X)[0].astype(np.float64)
    T = family.final_time(instance)
    t = family.plain_guess(instance)[0] if n_nodes is None else np.linspace(0.0, T, n_nodes)
    y, z, p = guess_from_vector(v, t, T, family.ny, family.nz, family.np)
    return bvpdae_write_data(path, len(t), family.ny, family.nz, family.np, t, y, z, p)


def write_solution_files(batch, path_fmt, device=True):
    """Every instance's solution of a solved Batch as a BVPDAEReadWriteData
    file: path_fmt % b names instance b's file.  device: the text is
    formatted on the GPU (Batch.solution_text, the same bytes), else by the
    host writer value by value.  Returns the list of writer statuses (0 ok,
    1 failure, as the reference's writer)."""
    if not device:
        from .io import bvpdae_write_data
        cp = batch.cp
        return [bvpdae_write_data(path_fmt % b, s["N"], cp.ny, cp.nz, cp.np, s["t"], s["y"], s["z"], s["p"])
                for b, s in enumerate(batch.solution())]
    text, off = batch.solution_text()
    out = []
    for b in range(batch.B):
        try:
            with open(path_fmt % b, "wb") as f:
                f.write(text[off[b]:off[b + 1]])
            out.append(0)
        except OSError:
            out.append(1)
    return out


def pack_family(family, instances):
    """Packed host arrays (N, t, y, z, p, theta) of the plain guesses."""
    parts = [family.plain_guess(i) for i in instances]
    N = np.array([len(p[0]) for p in parts], dtype=np.int32)
    t = np.concatenate([p[0] for p in parts])
    y = np.concatenate([p[1] for p in parts])
    z = np.concatenate([p[2] for p in parts]) if family.nz else np.zeros((int(N.sum()), 0))
    p = np.array([pp[3] for pp in parts]).reshape(len(instances), -1)
    th = np.array([family.theta(i) for i in instances]).reshape(len(instances), -1)
    return N, t, y, z, p, th


class BatchSolver:
    """Solves lists of instances of a family in one batch per m; compiled
    problems are kept per m, and idle batches per (m, instance count), so a
    repeated solve of as many instances (the fallbacks of a warm-started
    batch) sets its guesses into device buffers it already has instead of
    allocating and freeing them (cudaFree waits for the whole device)."""

    _KEEP = 8  # idle batches kept, least recently used dropped first

    def __init__(self, family, opts=None, layout=0):
        self.family = family
        self.compiled = {}
        self.layout = layout
        self.opts = opts if opts is not None else default_opts(family.problem, max_nodes=20000)
        self._idle = collections.OrderedDict()
        self._lock = threading.Lock()

    def _take(self, m, n):
        with self._lock:
            free = self._idle.get((m, n))
            if free:
                self._idle.move_to_end((m, n))
                return free.pop()
        return Batch(self.cp(m), n)

    def batches(self):
        """The idle batches kept for reuse (their profile counters count the
        launches of the solves they ran)."""
        with self._lock:
            return [bt for v in self._idle.values() for bt in v]

    def _give(self, m, n, bt):
        with self._lock:
            self._idle.setdefault((m, n), []).append(bt)
            self._idle.move_to_end((m, n))
            while sum(len(v) for v in self._idle.values()) > self._KEEP:
                k, v = next(iter(self._idle.items()))
                v.pop(0)
                if not v:
                    del self._idle[k]

    def cp(self, m):
        if m not in self.compiled:
            self.compiled[m] = CompiledProblem(self.family.problem, m, layout=self.layout)
        return self.compiled[m]

    def solve(self, instances, guesses=None):
        """Solve every instance (guesses: list of (y, z, p) on the plain mesh or
        None for the plain guess).  Returns the solution dicts in input order."""
        fam = self.family
        out = [None] * len(instances)
        for m in sorted(set(i.m for i in instances)):
            idx = [k for k, i in enumerate(instances) if i.m == m]
            meshes, ps, ths = [], [], []
            for k in idx:
                inst = instances[k]
                t, y0, z0, p0 = fam.plain_guess(inst)
                if guesses is not None and guesses[k] is not None:
                    y0, z0, p0 = guesses[k]
                meshes.append((t, y0, z0))
                ps.append(p0)
                ths.append(fam.theta(inst))
            bt = self._take(m, len(idx))
            bt.set_guess(meshes, np.array(ps).reshape(len(idx), -1), np.array(ths).reshape(len(idx), -1))
            bt.solve(self.opts)
            for k, s in zip(idx, bt.solution()):
                out[k] = s
            self._give(m, len(idx), bt)
        return out


def training_set(family, solver, instances):
    """(X, Y) from the instances the batched solver solves from the plain guess."""
    sols = solver.solve(instances)
    X, Y = [], []
    for inst, s in zip(instances, sols):
        if not s["success"]:
            continue
        X.append(family.features(inst))
        Y.append(trajectory_vector(s["t"], s["y"], s["z"], s["p"], family.final_time(inst)))
    return np.array(X, np.float32), np.array(Y, np.float32), sols


def warm_guesses(family, mlp, instances):
    X = np.array([family.features(i) for i in instances], np.float32)
    pred = mlp.predict(X).astype(np.float64)
    out = []
    for inst, v in zip(instances, pred):
        t = family.plain_guess(inst)[0]
        out.append(guess_from_vector(v, t, family.final_time(inst), family.ny, family.nz, family.np))
    return out


def solve_warm(family, solver, mlp, instances):
    """Warm-started batch solve with fallback: instances whose warm-started
    solve fails are solved again from the plain guess.  Returns (solutions,
    fallback indices, warm-start solutions)."""
    guesses = warm_guesses(family, mlp, instances)
    warm = solver.solve(instances, guesses)
    fb = [k for k, s in enumerate(warm) if not s["success"]]
    final = list(warm)
    if fb:
        plain = solver.solve([instances[k] for k in fb])
        for k, s in zip(fb, plain):
            s = dict(s)
            s["fallback"] = True
            final[k] = s
    return final, fb, warm


class WarmRunner:
    """Device-resident warm-started batch solve of a fixed list of instances:
    features and plain guesses live in HBM; each run resets the batches,
    predicts the trajectories, fills the guesses on the device, solves, and
    solves the failed instances again from the plain guess.

    spares: each m-group's batch also holds every instance a second time
    from the plain guess, paired with its warm-started copy (Batch.set_spares):
    the fallback solves then run inside the warm solve's own super-steps
    instead of after it."""

    def __init__(self, family, solver, mlp, instances, spares=False):
        from .module import DeviceArray
        self.family, self.solver, self.mlp = family, solver, mlp
        self.spares = bool(spares)
        order = sorted(range(len(instances)), key=lambda k: instances[k].m)
        self.instances = [instances[k] for k in order]
        self.order = order
        X = np.array([family.features(i) for i in self.instances], np.float32)
        self.dX = DeviceArray(X.shape, np.float32)
        self.dX.upload(X)
        self.dY = DeviceArray((len(self.instances), mlp.n_out), np.float32)
        self.groups = []
        start = 0
        for m in sorted(set(i.m for i in self.instances)):
            idx = [k for k, i in enumerate(self.instances) if i.m == m]
            assert idx == list(range(start, start + len(idx)))
            meshes, ps, ths = [], [], []
            for k in idx:
                t, y0, z0, p0 = family.plain_guess(self.instances[k])
                meshes.append((t, y0, z0))
                ps.append(p0)
                ths.append(family.theta(self.instances[k]))
            n = len(idx)
            copies = 2 if self.spares else 1
            bt = Batch(solver.cp(m), copies * n)
            bt.set_guess(meshes * copies, np.array(ps * copies).reshape(copies * n, -1),
                         np.array(ths * copies).reshape(copies * n, -1))
            if self.spares:
                bt.set_spares(n, -1)
            self.groups.append(dict(m=m, first=start, n=n, bt=bt))
            start += len(idx)

    def run(self, warm=True, fallback=True, threads=True, speculate=0.0, spare_at=0.02):
        """One solve of every instance; returns (solved, fallback count, stats).
        self.times holds the seconds of the phases of the last run.

        spare_at (runners built with spares): the spares start once no more
        than this fraction of a group is in the Newton iteration.  Every
        instance's result is independent of its batch-mates and of when its
        spare started, so the outcome is the one of falling back after the
        warm solve.

        speculate: once no more than this fraction of a group is still in the
        Newton iteration, the instances still iterating are solved from the
        plain guess on a second thread while the warm solve goes on; an
        instance that then fails from its warm guess takes that solution,
        one that succeeds drops it.  Each instance's result is independent
        of its batch-mates, so the outcome is the one of solving the failed
        instances again afterwards; only the wall time changes.  0 (the
        default) falls back after the warm solve: on the Van der Pol batch
        the overlapped chains of small launches contend for the GPU and the
        step is slower (0.66 s against 0.55 s at 0.03)."""
        import threading
        import time
        t0 = time.perf_counter()
        if warm:
            self.mlp.predict_device(self.dX, len(self.instances), self.dY)
        t1 = time.perf_counter()

        def plain_solve(g, ks):
            return self.solver.solve([self.instances[g["first"] + k] for k in ks])

        def one(g):
            bt = g["bt"]
            if self.spares:
                bt.set_spares(g["n"], max(0, int(spare_at * g["n"])) if warm and fallback else -1)
            bt.reset()
            if warm:
                bt.warm_start(self.dY.ptr + 4 * g["first"] * self.mlp.n_out, N_NODES, self.mlp.n_out)
            spec = {}
            if warm and fallback and speculate > 0 and not self.spares:
                limit = max(1, int(speculate * g["n"]))

                def side(ks):
                    try:
                        spec["sols"] = plain_solve(g, ks)
                    except BaseException as e:  # re-raised on the group's thread
                        spec["error"] = e

                def hook(active, steps):
                    if "ks" in spec or active > limit:
                        return
                    st = bt.statuses()
                    spec["ks"] = [int(k) for k in np.flatnonzero((st == 0) | (st == 1))]
                    spec["t"] = time.perf_counter() - t1
                    if spec["ks"]:
                        spec["thread"] = threading.Thread(target=side, args=(spec["ks"],))
                        spec["thread"].start()
                bt.set_progress(hook)
            try:
                bt.solve(self.solver.opts)
            except BaseException:
                if "thread" in spec:
                    spec["thread"].join()
                raise
            finally:
                bt.set_progress(None)
            g["t_solve"] = time.perf_counter() - t1
            if self.spares:
                n = g["n"]
                packed = bt.solution_packed()
                st = np.ctypeslib.as_array(packed[5])["status"]
                failed = [int(k) for k in np.flatnonzero(st[:n] != 3)] if warm and fallback else []
                for k in failed:
                    if st[n + k] not in (3, 4):
                        raise RuntimeError("spare of failed instance %d did not run (status %d)" % (k, st[n + k]))
                sols = bt.solution(list(range(n)) + [n + k for k in failed], packed=packed)
                g["sols"] = sols[:n]
                for j, k in enumerate(failed):
                    g["sols"][k] = dict(sols[n + j], fallback=True)
                g["fallback"] = failed
                g["speculated"] = int(np.count_nonzero(st[n:] != 6))
                g["t_spec"] = None
                g["t_done"] = time.perf_counter() - t1
                return
            g["sols"] = bt.solution()
            if "thread" in spec:
                spec["thread"].join()
            g["fallback"] = []
            g["speculated"] = len(spec.get("ks", []))
            g["t_spec"] = spec.get("t")
            if "error" in spec:
                raise spec["error"]
            if warm and fallback:
                # (a second thread for these solves while this one downloads
                # the batch's solutions was measured slower: 0.574 s per step
                # against 0.553 s)
                failed = [k for k, s in enumerate(g["sols"]) if not s["success"]]
                have = dict(zip(spec.get("ks", []), spec.get("sols", [])))
                rest = [k for k in failed if k not in have]
                if rest:
                    have.update(zip(rest, plain_solve(g, rest)))
                for k in failed:
                    g["sols"][k] = dict(have[k], fallback=True)
                g["fallback"] = failed
            g["t_done"] = time.perf_counter() - t1

        if threads:
            ths = [threading.Thread(target=one, args=(g,)) for g in self.groups]
            for t in ths:
                t.start()
            for t in ths:
                t.join()
        else:
            for g in self.groups:
                one(g)
        t2 = time.perf_counter()
        sols = []
        n_fb = 0
        for g in self.groups:
            sols += g["sols"]
            n_fb += len(g["fallback"])
        self.times = {"predict_s": t1 - t0, "solve_and_fallback_s": t2 - t1,
                      "groups": [(g["m"], round(g["t_solve"], 4), round(g["t_done"], 4)) for g in self.groups],
                      "speculated": [(g["m"], g["speculated"], None if g["t_spec"] is None else round(g["t_spec"], 4))
                                     for g in self.groups]}
        solved = sum(int(s["success"]) for s in sols)
        return solved, n_fb, sols
