"""Benchmark: solves per second to a 1e-6 residual on one GB300 (FP64):
NN-warm-started batched solves against the plain GPU solver on the same
batch, with the CPU oracle timed beside them.

Default workload (`--workload warm`, the learned-warm-start configuration):
the Van der Pol family (x0 ~ U[-2,2]^2, T ~ U[2,8], control weight
r ~ logU[0.1,10]).  Set-up (untimed, reported): 65,536 seeded instances
(seed 1000, N ~ U{32..256} intervals) solved by the batched solver from the
plain guess, an MLP (4 layers, width 256, GELU, BF16 operands, FP32
accumulation) trained on them by the library's kernels.  One "step": the
8192 held-out instances (seed 7, N ~ U{32..2048} intervals, m ~ U{3,4,5})
solved to completion in one batch per m: features -> MLP -> trajectories
interpolated onto each mesh (on the device) -> Newton, line search, segment
residual, remesh; instances whose warm-started solve fails are solved again
from the plain guess.

  value  solves/s (instances reaching the tolerance), inputs resident in HBM
  e2e    the same through the C ABI from pinned host buffers: features and
         plain guesses H2D, solutions D2H, inside the timed region (one host
         thread per m-group, as for value)
  plain_batched      the same batch from the plain (zero) guess
  plain_single_gpu   the plain solver one instance at a time (a random sample)

`--workload plain`: the batched plain solve of 4096 instances (seed 1,
N ~ U{32..2048}) alone.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank solves its own batch (seeds + rank; weak scaling)
and rank 0 prints one JSON line.
"""
import argparse
import importlib
import json
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "collocation-solver-cuda_gb300"
METRIC = "solves/sec to 1e-6 residual: NN-warm-started batched vs plain GPU, same GB300"
BATCH = 4096
SEED = 1
BABD_PATH = [0]


def _pkg():
    return importlib.import_module(PKG)


_T_START = time.time()


def _log(msg):
    """Progress on stderr (the JSON line goes to stdout)."""
    print("[bench %7.1f s] %s" % (time.time() - _T_START, msg), file=sys.stderr, flush=True)


# ------------------------------------------------------------ CPU oracle ---
_WORKER_PROBLEMS = {}


def _family(cs, name):
    ws = cs.warmstart
    return ws.vdp_family() if name == "vdp" else ws.pendulum_family(8)


def _family_batch(cs, name, n, seed, train=False):
    """Seeded instances of a warm-start family (training draws use shorter meshes)."""
    if name == "vdp":
        return cs.workloads.vdp_batch(n, seed=seed, n_range=(32, 256) if train else (32, 2048))
    return cs.workloads.pendulum_batch(n, K=8, seed=seed, n_range=(32, 128))


def _inst_args(family, inst):
    if family == "vdp":
        return (family, tuple(inst.x0), inst.T, inst.r, inst.intervals, inst.m)
    return (family, tuple(inst.theta0), inst.T, inst.k, inst.intervals, inst.m)


def _oracle_worker(args):
    """Solve one instance with the CPU oracle (runs in a spawned process;
    a = None only prepares the problem)."""
    family, a, T, c, intervals, m = args
    cs = _pkg()
    from oracle import collocation_oracle as O
    if family not in _WORKER_PROBLEMS:
        fam = _family(cs, family)
        pr = fam.problem

        class P:
            pass

        op = P()
        op.__dict__.update(pr.__dict__)
        op.ny, op.nz, op.np = pr.size_y, pr.size_z, pr.size_p
        nf = cs.codegen.NumpyProblem(cs.codegen.ProblemCode(pr.sym))
        for k in ("f", "g", "Df", "Dg", "r", "Dr"):
            setattr(op, k, getattr(nf, k))
        _WORKER_PROBLEMS[family] = (fam, op)
    fam, op = _WORKER_PROBLEMS[family]
    if a is None:
        return None
    if family == "vdp":
        inst = cs.workloads.VdpInstance(np.array(a), T, c, intervals, m)
    else:
        inst = cs.workloads.PendulumInstance(np.array(a), T, c, intervals, m)
    op.theta = fam.theta(inst)
    t, y, z, p = fam.plain_guess(inst)
    res = O.solve(op, m, cs.tables.lobatto(m), cs.tables.segment_tables(m), T0=t, Y0=y, Z0=z, P0=p)
    return res.success, res.N


def _oracle_prepare(family):
    """Import, derivation and numpy code generation in a worker (no solve)."""
    return _oracle_worker((family, None, 0.0, 0.0, 0, 0))


class OracleSampler:
    """A pool of single-threaded oracle processes (spawned, BLAS pinned to
    one thread each before numpy loads in the children) that solves
    instances for a bounded wall-clock window."""

    ENV = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")

    def __init__(self, family, procs):
        self.family, self.procs = family, procs
        saved = {k: os.environ.get(k) for k in self.ENV}
        for k in self.ENV:
            os.environ[k] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(procs)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        self.pool.map(_oracle_prepare, [family] * procs)

    def run(self, instances, window_s, grace_s=30.0):
        """Solve instances in order, `procs` at a time, starting new ones
        until `window_s` has passed; returns (completed, seconds from the
        start to the last completion).  Solves still running `grace_s` after
        the window are abandoned (the sample then favours the CPU)."""
        it = iter([_inst_args(self.family, i) for i in instances])
        pending = []
        t0 = time.time()
        t_last = t0
        done = 0

        def submit():
            a = next(it, None)
            if a is not None:
                pending.append(self.pool.apply_async(_oracle_worker, (a,)))

        for _ in range(self.procs):
            submit()
        while pending:
            for r in [r for r in pending if r.ready()]:
                pending.remove(r)
                r.get()
                done += 1
                t_last = time.time()
                if t_last - t0 < window_s:
                    submit()
            if time.time() - t0 > window_s + grace_s:
                break
            time.sleep(0.005)
        self.abandoned = len(pending)
        return done, max(t_last - t0, 1e-9)

    def close(self):
        self.pool.terminate()
        self.pool.join()


def cpu_oracle_rate(instances, procs, target_s=20.0, family="vdp"):
    """Solves/s of the oracle on a bounded sample, with `procs` processes."""
    smp = OracleSampler(family, procs)
    try:
        done, dt = smp.run(instances, target_s)
    finally:
        smp.close()
    return done / dt, done, dt


# --------------------------------------------------------------- clocks ---
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def fp64_peak_with_clock(cs, gpu, seconds=1.0):
    """The DFMA peak (best of repeated runs of cs_measure_fp64_peak over
    about `seconds`) with the SM clock sampled while it runs, so that the
    roofline denominator is pinned to the clock it was measured at; also the
    FP64 tensor-core (DMMA) rate for comparison."""
    vals = []
    with ClockSampler(gpu) as clk:
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds or len(vals) < 3:
            vals.append(cs.module.measure_fp64_peak())
    summ = clk.summary()
    return max(vals), {"tflops_runs": len(vals), "sm_mhz": summ.get("sm_mhz"), "sm_max_mhz": summ.get("sm_max_mhz"),
                       "reasons": summ.get("reasons"), "dmma_tflops": cs.module.measure_dmma_peak()}


# ------------------------------------------------------------ GPU batch ---
class Workload:
    """The batch split by m, one compiled problem and one Batch per group."""

    def __init__(self, cs, instances):
        self.cs = cs
        self.problem = cs.workloads.vdp_family_problem()
        self.groups = []
        for m in sorted(set(i.m for i in instances)):
            insts = [i for i in instances if i.m == m]
            cp = cs.CompiledProblem(self.problem, m)
            N, t, y, z, p, th = cs.workloads.pack_vdp(insts)
            bt = cs.Batch(cp, len(insts), node_capacity=int(N.sum() * 2))
            host = {}
            for k, a in (("N", N), ("t", t), ("y", y), ("z", z), ("p", p), ("th", th)):
                pa = cs.module.PinnedArray(a.shape, a.dtype)
                pa.array[...] = a
                host[k] = pa
            cap = int(N.sum() * 4)
            out = {k: cs.module.PinnedArray(shape) for k, shape in
                   (("t", (cap,)), ("y", (cap, cp.ny)), ("z", (cap, max(cp.nz, 1))), ("p", (len(insts), cp.np)))}
            bt.set_guess_packed(host["N"].array, host["t"].array, host["y"].array, host["z"].array,
                                host["p"].array, host["th"].array)
            self.groups.append(dict(m=m, insts=insts, cp=cp, bt=bt, host=host, out=out))
        self.opts = cs.default_opts(self.problem, max_nodes=20000, babd_path=BABD_PATH[0])
        self.n = len(instances)

    def _run_groups(self, fn):
        errs = []

        def wrap(g):
            try:
                fn(g)
            except Exception as e:  # noqa: BLE001
                errs.append(e)

        ths = [threading.Thread(target=wrap, args=(g,)) for g in self.groups]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        if errs:
            raise errs[0]

    def step_resident(self, threads=True):
        def f(g):
            g["bt"].reset()
            g["bt"].solve(self.opts)
        if threads:
            self._run_groups(f)
        else:
            for g in self.groups:
                f(g)

    def step_e2e(self):
        def f(g):
            h, o, bt = g["host"], g["out"], g["bt"]
            bt.set_guess_packed(h["N"].array, h["t"].array, h["y"].array, h["z"].array, h["p"].array, h["th"].array)
            bt.solve(self.opts)
            N, T = bt.sizes()
            if T > o["t"].array.shape[0]:
                raise RuntimeError("solution larger than the pinned output buffers")
            st = (self.cs._lib.Stats * bt.B)()
            self.cs._lib.check(bt._lib.cs_get_solution(bt.handle, self.cs._lib.dptr(o["t"].array),
                                                       self.cs._lib.dptr(o["y"].array), self.cs._lib.dptr(o["z"].array),
                                                       self.cs._lib.dptr(o["p"].array), st), "cs_get_solution")
            g["last_T"] = T
            g["last_stats"] = st
        self._run_groups(f)

    def h2d_bytes(self):
        return int(sum(sum(h.array.nbytes for h in g["host"].values()) for g in self.groups))

    def d2h_bytes(self):
        tot = 0
        for g in self.groups:
            T = g.get("last_T", 0)
            cp = g["cp"]
            tot += 8 * T * (1 + cp.ny + cp.nz) + 8 * g["bt"].B * cp.np + g["bt"].B * 64
        return int(tot)

    def results(self):
        succ, newton, N = 0, 0, 0
        for g in self.groups:
            for s in g["bt"].solution():
                succ += int(s["success"])
                newton += s["newton_steps"]
                N += s["N"]
        return succ, newton, N


# DRAM bytes per condensed interval measured by ncu per m, one launch over
# about a million intervals of each m-group (working set far above L2:
# dram__bytes_read.sum + dram__bytes_write.sum ÷ intervals,
# profiles/k_condense_vdp_batch3072_mix.md)
TRAFFIC_PER_INTERVAL_NCU = {3: 1000.4, 4: 1240.4, 5: 1474.0}


def flops_per_interval(m, ny=4, nz=1, npe=0):
    """Algorithmic FP64 flops of condensing one interval: (2/3) s^3 + 2 s^2 r,
    s = m (ny + nz), r = ny + np_eff + 1 (LU of the stage system with r
    right-hand sides and their back substitution)."""
    s = m * (ny + nz)
    r = ny + npe + 1
    return 2.0 / 3.0 * s ** 3 + 2.0 * s * s * r


def bytes_per_interval(m, ny=4, nz=1, npe=0):
    """Algorithmic HBM bytes of condensing one interval: read t, y_i, y_{i+1},
    y', z~; write X = W^-1 [J V f_a] and the block row [A C H b]."""
    s = m * (ny + nz)
    r = ny + npe + 1
    return 8 * (2 + 2 * ny + m * (ny + nz) + r * s + ny * (2 * ny + npe + 1))


def _rank_device(env, local_rank, world):
    """CUDA_VISIBLE_DEVICES for a rank under torchrun: its own GPU among the
    visible ones (the library works on the current device, so each rank sees
    exactly one)."""
    if world <= 1:
        return env.get("CUDA_VISIBLE_DEVICES")
    vis = env.get("CUDA_VISIBLE_DEVICES")
    devs = [d for d in vis.split(",") if d.strip()] if vis else [str(i) for i in range(world)]
    return devs[local_rank % len(devs)]


_GPU_ID = [None]


def _gpu_index(local_rank):
    """nvidia-smi index of this rank's GPU (physical, from CUDA_VISIBLE_DEVICES)."""
    return _GPU_ID[0] if _GPU_ID[0] is not None else local_rank


def _dist_setup(world, local_rank):
    if world <= 1:
        return None
    import torch.distributed as tdist
    tdist.init_process_group("gloo")
    return tdist


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def _roofline(groups, fp64_peak):
    """Condensation of every interval of each group, timed alone with CUDA
    events on the batch's stream (one launch per group)."""
    flops = cbytes = cms = traffic = 0.0
    n_all = 0
    for m, bt in groups:
        bt.reset()
        ms = bt.time_condense(reps=5)
        n_int = bt.sizes()[1] - bt.B
        cp = bt.cp
        flops += n_int * flops_per_interval(m, cp.ny, cp.nz, cp.np_eff)
        cbytes += n_int * bytes_per_interval(m, cp.ny, cp.nz, cp.np_eff)
        cms += ms
        n_all += n_int
        # measured for the Van der Pol family only (ny = 4)
        traffic += (TRAFFIC_PER_INTERVAL_NCU.get(m, float("nan")) if cp.ny == 4 else float("nan")) * n_int
    achieved = flops / (cms * 1e-3) / 1e12
    return {"bound": "fp64", "kernel": "k_condense", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": achieved / fp64_peak if fp64_peak else None,
            "traffic": (traffic / len(groups)) if traffic == traffic else None,
            "traffic_note": "DRAM bytes per launch (average over the m-groups): bytes per interval measured by ncu "
                            "for each m on a launch of ~1M intervals (profiles/k_condense_vdp_batch3072_mix.md: "
                            "1000 / 1240 / 1474 B for m = 3 / 4 / 5, 92-94 % of the algorithmic bytes) times the "
                            "intervals of this launch; algorithmic bytes per interval are in flops_note",
            "peak_source": "DFMA microbenchmark (cs_measure_fp64_peak) in this run, best of repeated runs over "
                           "about a second with the SM clock sampled meanwhile (peak_measurement); FP64 is absent "
                           "from MEASURED_PEAKS.json",
            "flops_per_launch": flops / len(groups), "ms_per_launch": cms / len(groups),
            "flops_note": "contract flops per interval (2/3)s^3 + 2 s^2 r, s = m(ny+nz), r = ny+np_eff+1; "
                          "algorithmic bytes 8(2 + 2ny + m(ny+nz) + r s + ny(2ny+np_eff+1)) per interval",
            "hbm_gbs": cbytes / (cms * 1e-3) / 1e9}


def _cpu_baseline(instances, cores, seed=3, family="vdp"):
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(instances))
    sample = [instances[i] for i in idx]
    rate, n, dt = cpu_oracle_rate(sample, cores, target_s=20.0, family=family)
    return {"value": rate, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": "%d random instances of the batch solved by the oracle from the plain guess in %.1f s, one "
                      "process per core (single-threaded BLAS)" % (n, dt)}


def run_reference(args, instances, cfg, cores):
    """The reference's CPU implementation of the path (its Python restated as
    the oracle), all host cores, one process per core; each step is a
    bounded sample: the instances that finish in a 10 s window."""
    sample = instances[:]
    rng = np.random.default_rng(7)
    rng.shuffle(sample)
    smp = OracleSampler(args.family, cores)
    window = 10.0
    pos = 0
    try:
        for _ in range(args.warmup):
            d, _ = smp.run(sample[pos:], window)
            pos += d + smp.abandoned
        done = 0
        t_all = 0.0
        wall0 = time.time()
        for _ in range(args.steps):
            d, dt = smp.run(sample[pos:], window)
            pos += d + smp.abandoned
            done += d
            t_all += dt
        wall = time.time() - wall0
    finally:
        smp.close()
    v = done / t_all
    cfg = dict(cfg, l2="n/a (CPU)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": "%d random instances of the batch from the plain guess (the reference has no "
                                       "warm start), one process per core, those finishing in a %.0f s window per "
                                       "step" % (done, window)},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_warm(args, cs, rank, world, local_rank, cpu, cfg):
    dist = _dist_setup(world, local_rank)
    cs.build.build_library()
    cs._lib.load()
    ws = cs.warmstart
    fp64_peak, peak_clock = fp64_peak_with_clock(cs, _gpu_index(local_rank))
    fam = _family(cs, args.family)
    solver = ws.BatchSolver(fam, cs.default_opts(fam.problem, max_nodes=20000, babd_path=args.babd_path,
                                                  ls_grow=args.ls_grow), layout=args.layout)
    # ---- set-up: training data from the batched solver, then training
    t0 = time.perf_counter()
    train = _family_batch(cs, args.family, args.train, 1000 + 100 * rank, train=True)
    _log("training set: solving %d instances" % len(train))
    X, Y, _ = ws.training_set(fam, solver, train)
    t_data = time.perf_counter() - t0
    _log("training set: %d solutions in %.1f s; training" % (len(X), t_data))
    t0 = time.perf_counter()
    net = ws.Mlp(X.shape[1], Y.shape[1], width=args.width, depth=4, seed=0)
    net.fit_normalization(X, Y)
    loss = net.train(X, Y, epochs=args.epochs, batch=1024, lr=args.lr, seed=0,
                     lr_final=args.lr_final if args.lr_final >= 0 else None)
    t_train = time.perf_counter() - t0
    # ---- evaluation batch, resident in HBM
    _log("trained in %.1f s (loss %.3g)" % (t_train, loss))
    held = _family_batch(cs, args.family, args.batch, 7 + 100 * rank)
    runner = ws.WarmRunner(fam, solver, net, held, spares=args.spares >= 0)
    spare_at = max(args.spares, 0.0)
    # launch-shape tuner (set-up, untimed): condensation shape per m on the batch
    tune = [dict(m=g["m"], **g["bt"].autotune(reps=3)) for g in runner.groups]
    _log("tuned condensation shapes: %s" % tune)
    ws_gb = sum(g["bt"].sizes()[1] for g in runner.groups) * 8 * 300 / 1e9
    cfg["l2"] = cfg["l2"] % ("%.1f" % ws_gb)
    for _ in range(args.warmup):
        runner.run(warm=True, speculate=args.speculate, spare_at=spare_at)
    for bt in [g["bt"] for g in runner.groups] + solver.batches():
        bt.profile_reset(timing=False)
    _log("warm-up done; timed warm-started steps")
    _barrier(dist)
    with ClockSampler(_gpu_index(local_rank)) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            solved, n_fb, sols = runner.run(warm=True, speculate=args.speculate, spare_at=spare_at)
        dt = time.perf_counter() - t0
    dt = _max_over_ranks(dist, dt)
    runner_times = dict(runner.times)
    # the m-group batches, the fallback solves' batches, and the network's
    # 6 launches per step (input gather, 4 GEMMs, output scaling)
    launches = (sum(g["bt"].profile()["launches"] for g in runner.groups)
                + sum(bt.profile()["launches"] for bt in solver.batches()) + args.steps * 6)
    value = _sum_over_ranks(dist, args.steps * solved) / dt
    newton_warm = np.mean([s["newton_steps"] for s in sols])
    # ---- plain batched solve of the same instances
    _log("warm: %.1f solves/s; plain batched" % value)
    runner.run(warm=False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solved_p, _, sols_p = runner.run(warm=False)
    dtp = _max_over_ranks(dist, time.perf_counter() - t0)
    plain_batched = _sum_over_ranks(dist, args.steps * solved_p) / dtp
    newton_plain = np.mean([s["newton_steps"] for s in sols_p])
    # ---- plain one-instance GPU solver on a random sample of the same batch
    _log("plain batched: %.1f solves/s; plain one-instance sample" % plain_batched)
    rng = np.random.default_rng(11)
    sample = [held[k] for k in rng.choice(len(held), size=args.single_sample, replace=False)]
    solver.solve(sample[:2])
    t0 = time.perf_counter()
    n_ok = 0
    for inst in sample:
        n_ok += int(solver.solve([inst])[0]["success"])
    dts = time.perf_counter() - t0
    plain_single = n_ok / dts
    # ---- end to end through the C ABI from pinned host buffers
    _log("plain one-instance: %.1f solves/s; end to end" % plain_single)
    Xh = cs.module.PinnedArray((len(runner.instances), X.shape[1]), np.float32)
    Xh.array[...] = np.array([fam.features(i) for i in runner.instances], np.float32)
    hosts = []
    for g in runner.groups:
        insts = runner.instances[g["first"]:g["first"] + g["n"]]
        N, t, y, z, p, th = ws.pack_family(fam, insts * (2 if runner.spares else 1))
        hh = {}
        for k, a in (("N", N), ("t", t), ("y", y), ("z", z), ("p", p), ("th", th)):
            pa = cs.module.PinnedArray(a.shape, a.dtype)
            pa.array[...] = a
            hh[k] = pa
        cap = int(N.sum() * 4)
        out = {k: cs.module.PinnedArray(shape) for k, shape in (("t", (cap,)), ("y", (cap, fam.ny)),
                                                                 ("z", (cap, fam.nz)), ("p", (g["bt"].B, fam.np)))}
        hosts.append((hh, out))
    h2d = Xh.array.nbytes + sum(sum(a.array.nbytes for a in hh.values()) for hh, _ in hosts)
    d2h = 0
    def e2e_group(g, hh, out, res):
        # one m-group on its own host thread, as in the device-resident run:
        # guesses from pinned host memory, warm start, solve, solutions back to
        # pinned host memory, the failed instances again from the plain guess
        bt = g["bt"]
        n = g["n"]
        if runner.spares:
            bt.set_spares(n, int(spare_at * n))
        bt.set_guess_packed(hh["N"].array, hh["t"].array, hh["y"].array, hh["z"].array, hh["p"].array,
                            hh["th"].array)
        bt.warm_start(runner.dY.ptr + 4 * g["first"] * net.n_out, ws.N_NODES, net.n_out)
        bt.solve(solver.opts)
        Nn, T = bt.sizes()
        if T > out["t"].array.shape[0]:
            raise RuntimeError("solution larger than the pinned output buffers")
        st = (cs._lib.Stats * bt.B)()
        cs._lib.check(bt._lib.cs_get_solution(bt.handle, cs._lib.dptr(out["t"].array), cs._lib.dptr(out["y"].array),
                                              cs._lib.dptr(out["z"].array), cs._lib.dptr(out["p"].array), st),
                      "cs_get_solution")
        status = np.ctypeslib.as_array(st)["status"]
        d2h_fb = h2d_fb = 0
        if runner.spares:
            # a failed instance takes its spare's solution (started in the same solve)
            n_ok = int(np.count_nonzero((status[:n] == 3) | (status[n:] == 3)))
        else:
            # the failed instances again from the plain guess (host-built guesses
            # in, solutions out: counted with the step's bytes)
            failed = [runner.instances[g["first"] + b] for b in range(n) if status[b] != 3]
            n_ok = n - len(failed)
            for i, s in zip(failed, solver.solve(failed) if failed else []):
                n_ok += int(s["success"])
                d2h_fb += s["t"].nbytes + s["y"].nbytes + s["z"].nbytes + s["p"].nbytes + 64
                h2d_fb += sum(a.nbytes for a in fam.plain_guess(i)) + 8 * len(fam.theta(i))
        res[g["m"]] = (n_ok, 8 * T * (1 + fam.ny + fam.nz) + 8 * bt.B * fam.np + bt.B * 64 + d2h_fb, h2d_fb)

    _barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        runner.dX.upload(Xh.array)
        net.predict_device(runner.dX, len(runner.instances), runner.dY)
        res = {}
        ths = [threading.Thread(target=e2e_group, args=(g, hh, out, res)) for g, (hh, out) in zip(runner.groups, hosts)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        if len(res) != len(runner.groups):
            raise RuntimeError("end-to-end step: an m-group failed")
        n_e2e = sum(v[0] for v in res.values())
        d2h = sum(v[1] for v in res.values())
        h2d_fb = sum(v[2] for v in res.values())
    dte = _max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": _sum_over_ranks(dist, args.steps * n_e2e) / dte, "unit": "solves/s",
           "h2d_bytes_per_step": h2d + h2d_fb, "d2h_bytes_per_step": d2h}
    # ---- solution files of the whole batch: formatted on the GPU
    #      (cs_format_solutions) against the host writer on a sample
    files = _solution_files_rate(cs, runner)
    roof = _roofline([(g["m"], g["bt"]) for g in runner.groups], fp64_peak)
    roof["peak_measurement"] = peak_clock
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(),
                "gpu_launches": int(launches),
                "plain_batched": {"value": plain_batched, "unit": "solves/s", "solved": solved_p,
                                  "newton_steps_per_solve": float(newton_plain)},
                "plain_single_gpu": {"value": plain_single, "unit": "solves/s",
                                     "sample": "%d random instances of the batch, one Batch of 1 each" % len(sample)},
                "speedup_vs_plain_single_gpu": value / plain_single if plain_single else None,
                "solution_files": files,
                "warm_start": {"solved": solved, "of": len(held), "fallbacks": n_fb, "phase_s": runner_times,
                               "fallback_rate": n_fb / len(held), "newton_steps_per_solve": float(newton_warm),
                               "train_solutions": int(len(X)), "train_data_s": t_data, "train_s": t_train,
                               "train_loss": loss, "epochs": args.epochs, "lr": args.lr,
                               "lr_schedule": ("cosine to %g of lr" % args.lr_final) if args.lr_final >= 0 else "constant"},
                "autotune": tune}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_plain(args, cs, rank, world, local_rank, cpu, cfg, instances):
    dist = _dist_setup(world, local_rank)
    cs.build.build_library()
    cs._lib.load()
    fp64_peak = cs.module.measure_fp64_peak()
    W = Workload(cs, instances)
    tune = [dict(m=g["m"], **g["bt"].autotune(reps=3)) for g in W.groups]
    ws_gb = sum(g["bt"].sizes()[1] for g in W.groups) * 8 * 300 / 1e9
    cfg["l2"] = cfg["l2"] % ("%.1f" % ws_gb)
    for _ in range(args.warmup):
        W.step_resident()
    for g in W.groups:
        g["bt"].profile_reset(timing=False)
    _barrier(dist)
    with ClockSampler(_gpu_index(local_rank)) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            W.step_resident()
        dt = time.perf_counter() - t0
    dt = _max_over_ranks(dist, dt)
    succ, newton, nodes = W.results()
    launches = sum(g["bt"].profile()["launches"] for g in W.groups)
    value = _sum_over_ranks(dist, args.steps * succ) / dt
    roof = _roofline([(g["m"], g["bt"]) for g in W.groups], fp64_peak)
    _barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        W.step_e2e()
    dte = _max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": _sum_over_ranks(dist, args.steps * succ) / dte, "unit": "solves/s",
           "h2d_bytes_per_step": W.h2d_bytes(), "d2h_bytes_per_step": W.d2h_bytes()}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(),
                "gpu_launches": int(launches),
                "solve_stats": {"solved": succ, "of": W.n, "newton_steps_per_solve": newton / W.n,
                                "final_nodes_per_solve": nodes / W.n},
                "autotune": tune}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------ large single instances ---
def _pendulum_configs():
    return _pkg().workloads.PENDULUM_CHAINS


def pendulum_problem(cs, K):
    return cs.workloads.pendulum_chain_problem(K)


def executed_flops_per_interval(m, ny, nz, npe):
    """FP64 flops the structured condensation executes per interval: LU of
    the stage system without its stage-0 block (s1 = (m-1)(ny+nz) rows) with
    r right-hand sides, their back substitution, and the stage-0 coupling of
    the right-hand sides (2 s1 r ny)."""
    s1 = (m - 1) * (ny + nz)
    r = ny + npe + 1
    return 2.0 / 3.0 * s1 ** 3 + 2.0 * s1 * s1 * r + 2.0 * s1 * r * ny


def _cpu_pendulum(cs, pr, m, slice_intervals=256):
    """The oracle (numpy, BLAS threads on all host cores) on one residual and
    one Newton step of the first `slice_intervals` intervals of the mesh;
    seconds per interval of each."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle import collocation_oracle as O

    class P:
        pass

    op = P()
    op.__dict__.update(pr.__dict__)
    op.ny, op.nz, op.np = pr.size_y, pr.size_z, pr.size_p
    nf = cs.codegen.NumpyProblem(cs.codegen.ProblemCode(pr.sym))
    for k in ("f", "g", "Df", "Dg", "r", "Dr"):
        setattr(op, k, getattr(nf, k))
    n = slice_intervals + 1
    t = np.asarray(pr.T0, float)[:n]
    rk = cs.tables.lobatto(m)
    y, yd, zt = O.form_initial_input(op, m, n, np.asarray(pr.Y0, float)[:n], np.asarray(pr.Z0, float)[:n],
                                     np.asarray(pr.P0, float), rk)
    p = np.asarray(pr.P0, float)
    t0 = time.time()
    f_q, y_tilde, f_a, f_b, r_bc = O.compute_f_q(op, m, n, rk, t, y, yd, zt, p, 0.1)
    t_res = time.time() - t0
    t0 = time.time()
    O.newton_step(op, m, n, rk, t, y, yd, zt, p, 0.1, f_a, f_b, r_bc, y_tilde)
    t_newton = time.time() - t0
    return t_res / slice_intervals, t_newton / slice_intervals


def run_pendulum_reference(args, cs, cores):
    """The reference's algorithm (the oracle port, numpy with BLAS on all
    cores) on the pendulum workload: a whole solve is minutes, so each step
    is one residual and one Newton step on 256 intervals, scaled to the
    full mesh and the solve's counts (3 Newton steps, 7 residuals, as the
    GPU solve of this configuration takes)."""
    c = _pendulum_configs()[args.pendulum]
    pr = pendulum_problem(cs, args.pendulum)
    n_int = c["nodes"] - 1
    for _ in range(args.warmup):
        _cpu_pendulum(cs, pr, c["m"])
    t0 = time.time()
    ts = [_cpu_pendulum(cs, pr, c["m"]) for _ in range(args.steps)]
    wall = time.time() - t0
    t_res = float(np.mean([a for a, _ in ts]))
    t_nw = float(np.mean([b for _, b in ts]))
    t_solve = 3 * t_nw * n_int + 7 * t_res * n_int
    v = 1.0 / t_solve
    line = {"impl": "reference", "metric": "solves/sec to %g residual: one large instance (pendulum chain K=%d), "
                                            "plain GPU solver" % (c["tol"], args.pendulum),
            "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "pendulum chain K=%d, Nodes=%d, m=%d" % (args.pendulum, c["nodes"], c["m"])},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": "one residual + one Newton step on 256 intervals per step, scaled"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_pendulum(args, cs, rank, world, local_rank):
    """One large instance per step (pendulum chain, FP64): solves/s, e2e from
    host buffers, roofline of the condensation, the oracle extrapolated."""
    K = args.pendulum
    c = _pendulum_configs()[K]
    m, nodes = c["m"], c["nodes"]
    cores = os.cpu_count() or 1
    pr = pendulum_problem(cs, K)
    cpu_t = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu_t = _cpu_pendulum(cs, pr, m)
    dist = _dist_setup(world, local_rank)
    cs.build.build_library()
    cs._lib.load()
    fp64_peak = cs.module.measure_fp64_peak()
    cp = cs.CompiledProblem(pr, m, precision=args.precision)
    bt = cs.Batch(cp, 1, node_capacity=4 * nodes)
    T0 = cs.module.PinnedArray((nodes,), np.float64)
    T0.array[...] = np.asarray(pr.T0, float)
    Y0 = cs.module.PinnedArray((nodes, cp.ny), np.float64)
    Y0.array[...] = np.asarray(pr.Y0, float)
    Z0 = cs.module.PinnedArray((nodes, cp.nz), np.float64)
    Z0.array[...] = np.asarray(pr.Z0, float)
    P0 = cs.module.PinnedArray((1, cp.np), np.float64)
    P0.array[...] = np.asarray(pr.P0, float)
    Nh = cs.module.PinnedArray((1,), np.int32)
    Nh.array[...] = nodes
    bt.set_guess_packed(Nh.array, T0.array, Y0.array, Z0.array, P0.array, None)
    opts = cs.default_opts(pr)
    tune = bt.autotune(reps=2)
    for _ in range(args.warmup):
        bt.reset()
        bt.solve(opts)
    bt.profile_reset(timing=False)
    _barrier(dist)
    with ClockSampler(_gpu_index(local_rank)) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            bt.reset()
            bt.solve(opts)
        dt = _max_over_ranks(dist, time.perf_counter() - t0)
    sol = bt.solution()[0]
    launches = bt.profile()["launches"]
    ok = int(sol["success"])
    value = _sum_over_ranks(dist, args.steps * ok) / dt
    # phases (one extra solve with per-launch event timing)
    bt.reset()
    bt.profile_reset(timing=True)
    bt.solve(opts)
    prof = bt.profile()
    bt.profile_reset(timing=False)
    # end to end: guess from pinned host memory, solution back to pinned memory
    cap = 4 * nodes
    out = {k: cs.module.PinnedArray(sh) for k, sh in (("t", (cap,)), ("y", (cap, cp.ny)), ("z", (cap, cp.nz)),
                                                       ("p", (1, cp.np)))}
    _barrier(dist)
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(args.steps):
        bt.set_guess_packed(Nh.array, T0.array, Y0.array, Z0.array, P0.array, None)
        bt.solve(opts)
        Nn, T = bt.sizes()
        st = (cs._lib.Stats * 1)()
        cs._lib.check(bt._lib.cs_get_solution(bt.handle, cs._lib.dptr(out["t"].array), cs._lib.dptr(out["y"].array),
                                              cs._lib.dptr(out["z"].array), cs._lib.dptr(out["p"].array), st),
                      "cs_get_solution")
        d2h = 8 * T * (1 + cp.ny + cp.nz) + 8 * cp.np + 64
    dte = _max_over_ranks(dist, time.perf_counter() - t0)
    h2d = T0.array.nbytes + Y0.array.nbytes + Z0.array.nbytes + P0.array.nbytes + Nh.array.nbytes
    e2e = {"value": _sum_over_ranks(dist, args.steps * ok) / dte, "unit": "solves/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}
    # roofline: one condensation of every interval of the final mesh
    bt.reset()
    ms = bt.time_condense(reps=3)
    n_int = nodes - 1
    fc = flops_per_interval(m, cp.ny, cp.nz, cp.np_eff)
    fe = executed_flops_per_interval(m, cp.ny, cp.nz, cp.np_eff)
    peak, bound = fp64_peak, "fp64"
    if args.precision != "fp64":
        # tensor-core condensation: against the measured dense BF16 peak
        try:
            peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"]
        except (OSError, KeyError, ValueError):
            peak = 1900.0
        bound = "tensor"
    roof = {"bound": bound, "kernel": "k_condense", "achieved": fc * n_int / (ms * 1e-3) / 1e12, "peak": peak,
            "unit": "TFLOP/s", "frac": fc * n_int / (ms * 1e-3) / 1e12 / peak, "traffic": None,
            "ms_per_launch": ms, "flops_per_launch": fc * n_int,
            "executed_tflops": fe * n_int / (ms * 1e-3) / 1e12,
            "executed_frac": fe * n_int / (ms * 1e-3) / 1e12 / fp64_peak,
            "flops_note": "achieved: contract flops (2/3)s^3 + 2 s^2 r per interval, s = m(ny+nz) = %d, r = %d; "
                          "executed: (2/3)s1^3 + 2 s1^2 r + 2 s1 r ny with s1 = (m-1)(ny+nz) = %d (the stage-0 "
                          "block is eliminated directly); peak of measured FP64 (DFMA microbenchmark, this run)"
                          % (m * (cp.ny + cp.nz), cp.ny + cp.np_eff + 1, (m - 1) * (cp.ny + cp.nz))}
    # reduced precision: max-abs difference from the FP64 solve of the same problem
    err = None
    if args.precision != "fp64":
        cp64 = cs.CompiledProblem(pr, m)
        b64 = cs.Batch(cp64, 1, node_capacity=4 * nodes)
        b64.set_guess_packed(Nh.array, T0.array, Y0.array, Z0.array, P0.array, None)
        b64.solve(opts)
        s64 = b64.solution()[0]
        if s64["N"] == sol["N"]:
            err = {"y": float(np.abs(sol["y"] - s64["y"]).max()), "z": float(np.abs(sol["z"] - s64["z"]).max()),
                   "p": float(np.abs(sol["p"] - s64["p"]).max()), "fp64_newton_steps": s64["newton_steps"]}
        else:
            err = {"note": "final meshes differ (%d vs %d nodes)" % (sol["N"], s64["N"])}
    cpu = None
    if cpu_t is not None:
        t_solve = sol["newton_steps"] * cpu_t[1] * n_int + sol["residual_evals"] * cpu_t[0] * n_int
        cpu = {"value": 1.0 / t_solve, "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": "oracle (numpy, BLAS on all cores) timed on one residual (%.2f ms/interval) and one Newton "
                         "step (%.2f ms/interval) of 256 intervals, scaled to the %d intervals and the %d Newton steps "
                         "and %d residuals of this solve" % (1e3 * cpu_t[0], 1e3 * cpu_t[1], n_int,
                                                              sol["newton_steps"], sol["residual_evals"])}
    if rank == 0:
        line = {"metric": "solves/sec to %g residual: one large instance (pendulum chain K=%d), plain GPU solver"
                          % (c["tol"], K),
                "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64 (%s condensation)" % args.precision,
                "data": "synthetic",
                "config": {"workload": "pendulum chain K=%d (ny %d, nz %d, np %d), Nodes=%d, m=%d, tol %g, "
                                       "theta(0)~U[-0.5,0.5] seed %d, guess theta_i(0)(1-t/T)"
                                       % (K, cp.ny, cp.nz, cp.np, nodes, m, c["tol"], c["seed"]),
                           "l2": "working set %.1f GB, larger than L2 (129 MB)"
                                 % (nodes * 8 * ((cp.ny + cp.np_eff + 1) * cp.s + 2 * cp.rowsz) / 1e9)},
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(),
                "gpu_launches": int(launches),
                "solve_stats": {"success": bool(sol["success"]), "N": sol["N"], "newton_steps": sol["newton_steps"],
                                "residual_evals": sol["residual_evals"], "max_residual": sol["max_residual"]},
                "phase_ms": {"condense": prof["condense_ms"], "babd": prof["babd_ms"],
                             "residual": prof["residual_ms"]},
                "precision": args.precision, "max_abs_error_vs_fp64": err, "autotune": tune}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def _solution_files_rate(cs, runner, sample=32):
    """Text of every instance's solution file (the reference's format) for the
    solved batch: formatted on the GPU, and by the host writer for a sample of
    instances, in bytes per second (untimed by the step)."""
    t0 = time.perf_counter()
    nbytes = 0
    for g in runner.groups:
        text, off = g["bt"].solution_text()
        nbytes += len(text)
    dt_dev = time.perf_counter() - t0
    g = runner.groups[0]
    sols = g["bt"].solution()[:sample]
    cp = g["bt"].cp
    t0 = time.perf_counter()
    hb = 0
    for s in sols:
        parts = ["nt:\n{}\nt:\n".format(s["N"]), "".join(cs.io._fmt(v) + " " for v in s["t"]),
                 "\nny:\n{}\ny:\n".format(cp.ny)]
        parts += ["".join(cs.io._fmt(v) + " " for v in row) + "\n" for row in s["y"]]
        parts.append("nz:\n{}\nz:\n".format(cp.nz))
        parts += ["".join(cs.io._fmt(v) + " " for v in row) + "\n" for row in s["z"]]
        parts.append("np:\n{}\np:\n".format(cp.np))
        parts.append("".join(cs.io._fmt(v) + " " for v in s["p"]))
        hb += len("".join(parts))
    dt_host = time.perf_counter() - t0
    return {"bytes": nbytes, "files": sum(g["bt"].B for g in runner.groups), "device_s": dt_dev,
            "device_MB_per_s": nbytes / dt_dev / 1e6, "host_MB_per_s": hb / dt_host / 1e6,
            "host_sample": "%d files of the m=%d group, Python writer (the reference's formatting)" % (len(sols), g["m"])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="warm", choices=["warm", "plain", "pendulum"])
    ap.add_argument("--family", default="vdp", choices=["vdp", "pendulum8"],
                    help="warm-start family (warm workload and its reference arm)")
    ap.add_argument("--pendulum", type=int, default=16, choices=[16, 32], help="chain length K (pendulum)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "tf32", "bf16", "tf32-tree", "bf16-tree"],
                    help="pendulum: precision of the large-system condensation")
    ap.add_argument("--batch", type=int, default=None, help="instances per step (warm: 8192, plain: 4096)")
    ap.add_argument("--train", type=int, default=65536, help="training solutions (warm)")
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--width", type=int, default=256, help="warm: hidden width of the MLP (4 layers)")
    ap.add_argument("--lr", type=float, default=2e-3, help="warm: Adam learning rate of the MLP")
    ap.add_argument("--lr-final", type=float, default=0.02,
                    help="warm: cosine decay of the learning rate to this fraction of it (negative: constant)")
    ap.add_argument("--single-sample", type=int, default=64)
    ap.add_argument("--speculate", type=float, default=0.0,
                    help="warm, without spares: start the plain-guess solves of the instances still iterating on "
                         "a second thread once at most this fraction of an m-group is (0: after the warm solve)")
    ap.add_argument("--spares", type=float, default=-1.0,
                    help="warm: the plain-guess copies of the instances ride in the warm batch and start once at "
                         "most this fraction of an m-group is in Newton, e.g. 0.005 (negative, the default: "
                         "separate fallback solves, 1-2 %% faster on the 8192-instance batch, where the GPU is busy "
                         "to the end of the step; the spares are ~10 %% faster on 2048)")
    ap.add_argument("--ls-grow", type=int, default=2,
                    help="line-search trials per super-step after a search that rejected k: ls_grow*k+2 "
                         "(0: all 20); same results")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--babd-path", type=int, default=0, help="0 automatic, 1 one CTA per instance, 2 per level")
    ap.add_argument("--layout", type=int, default=0,
                    help="kernel layout: 0 automatic, 1 shared-memory kernels, 2 large-system kernels")
    ap.add_argument("--profile-case", action="store_true",
                    help="small case for ncu: 512 instances, one full-batch condensation per m group, one solve; "
                         "with --workload pendulum: one Newton direction of the large instance")
    ap.add_argument("--profile-nodes", type=int, default=0,
                    help="pendulum profile case: nodes of the instance's mesh (0: the stated size)")
    ap.add_argument("--profile-instances", type=int, default=512,
                    help="instances of the plain profile case (the batched Van der Pol distribution, seed 1)")
    args = ap.parse_args()
    BABD_PATH[0] = args.babd_path
    if args.profile_case and args.workload == "pendulum":
        # one Newton direction of the large instance (for ncu)
        cs = _pkg()
        cs.build.build_library()
        lib = cs._lib.load()
        pr = cs.workloads.pendulum_chain_problem(args.pendulum, nodes=args.profile_nodes or None)
        cp = cs.CompiledProblem(pr, _pendulum_configs()[args.pendulum]["m"], precision=args.precision)
        bt = cs.Batch(cp, 1)
        bt.set_guess([(np.asarray(pr.T0, float), np.asarray(pr.Y0, float), np.asarray(pr.Z0, float))],
                     np.asarray(pr.P0, float).reshape(1, -1))
        cs._lib.check(lib.cs_profiler_start(), "cs_profiler_start")
        out = bt.stage_newton_direction(0.1)
        cs._lib.check(lib.cs_profiler_stop(), "cs_profiler_stop")
        print("profile case ok", float(np.abs(out["dy"]).max()))
        return
    if args.profile_case and args.workload == "warm":
        # one warm-started batch solve (2048 held-out instances, MLP trained on
        # 2048 solutions) inside the profiler range (cs_profiler_start/stop)
        cs = _pkg()
        cs.build.build_library()
        lib = cs._lib.load()
        ws = cs.warmstart
        fam = _family(cs, args.family)
        solver = ws.BatchSolver(fam, cs.default_opts(fam.problem, max_nodes=20000), layout=args.layout)
        X, Y, _ = ws.training_set(fam, solver, _family_batch(cs, args.family, 2048, 1000, train=True))
        net = ws.Mlp(X.shape[1], Y.shape[1], width=256, depth=4, seed=0)
        net.fit_normalization(X, Y)
        net.train(X, Y, epochs=args.epochs, batch=1024, lr=args.lr, seed=0,
                  lr_final=args.lr_final if args.lr_final >= 0 else None)
        runner = ws.WarmRunner(fam, solver, net, _family_batch(cs, args.family, 2048, 7), spares=args.spares >= 0)
        # the m-groups one after another on this thread (profilers serialise
        # kernels anyway, and a single host thread keeps the capture simple)
        runner.run(warm=True, threads=False, spare_at=max(args.spares, 0.0))
        cs._lib.check(lib.cs_profiler_start(), "cs_profiler_start")
        solved, n_fb, _ = runner.run(warm=True, threads=False, spare_at=max(args.spares, 0.0))
        cs._lib.check(lib.cs_profiler_stop(), "cs_profiler_stop")
        print("profile case ok: solved %d of 2048, %d fallbacks" % (solved, n_fb))
        return
    if args.profile_case:
        cs = _pkg()
        cs.build.build_library()
        W = Workload(cs, cs.workloads.vdp_batch(args.profile_instances, seed=SEED))
        for g in W.groups:
            g["bt"].reset()
            ms = g["bt"].time_condense(reps=1)
            print("m=%d condense %.3f ms over %d intervals" % (g["m"], ms, g["bt"].sizes()[1] - g["bt"].B))
        # the m-groups one after another on this thread: under ncu, solves
        # of several groups on several host threads ended the process with
        # error code 11 (the same run without ncu exits 0)
        W.step_resident(threads=False)
        # the solution files of the solved batch, formatted on the device
        nbytes = sum(len(g["bt"].solution_text()[0]) for g in W.groups)
        print("profile case ok", W.results(), "solution text %d bytes" % nbytes)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:  # before any CUDA call of this process
        dev = _rank_device(os.environ, local_rank, world)
        os.environ["CUDA_VISIBLE_DEVICES"] = dev
        _GPU_ID[0] = int(dev) if dev.isdigit() else local_rank
    else:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        first = vis.split(",")[0].strip() if vis else ""
        _GPU_ID[0] = int(first) if first.isdigit() else 0
    cs = _pkg()
    cores = os.cpu_count() or 1
    if args.workload == "pendulum":
        if args.impl == "reference":
            if rank == 0:
                run_pendulum_reference(args, cs, cores)
            return
        run_pendulum(args, cs, rank, world, local_rank)
        return
    if args.batch is None:
        args.batch = 8192 if args.workload == "warm" else BATCH
    if args.workload == "warm" and args.family == "pendulum8":
        instances = _family_batch(cs, "pendulum8", args.batch, 7 + 100 * rank)
        cfg = {"workload": "NN-warm-started batched solve: pendulum chain K=8 family (ny 32, nz 2, np 16), %d "
                           "held-out instances per GPU (theta(0)~U[-0.5,0.5]^8, T~U[5,15], k~U[0.2,1.0], "
                           "N~U{32..128} intervals, m=4, seed 7 + 100 rank), MLP trained on %d batched-solver "
                           "solutions (seed 1000)" % (args.batch, args.train),
               "batch_per_gpu": args.batch, "tol": 1e-6, "precision": "fp64 solver, bf16/fp32 network",
               "warm_start": "MLP 4x%d GELU, 64 normalised-time nodes, fallback to the plain guess" % args.width,
               "l2": "working set %s GB per step, larger than L2 (129 MB)"}
    elif args.workload == "warm":
        instances = cs.workloads.vdp_batch(args.batch, seed=7 + 100 * rank)
        cfg = {"workload": "NN-warm-started batched solve: Van der Pol family, %d held-out instances per GPU "
                           "(x0~U[-2,2]^2, T~U[2,8], r~logU[0.1,10], N~U{32..2048} intervals, m~U{3,4,5}, seed 7 + "
                           "100 rank), MLP trained on %d batched-solver solutions (seed 1000, N~U{32..256})"
                           % (args.batch, args.train),
               "batch_per_gpu": args.batch, "tol": 1e-6, "precision": "fp64 solver, bf16/fp32 network",
               "warm_start": "MLP 4x%d GELU, 64 normalised-time nodes, fallback to the plain guess" % args.width,
               "l2": "working set %s GB per step, larger than L2 (129 MB)"}
    else:
        cfg = None
    if cfg is not None:
        if args.spares >= 0:
            cfg["fallback"] = ("every instance that fails from its warm guess is solved again from the plain guess, "
                               "inside the same batch: each m-group batch holds every instance twice (warm and "
                               "plain copy); the plain copies of the instances still iterating or failed start "
                               "once at most %g of the group is in Newton, those whose warm copy succeeded stop "
                               "(same results as solving the failed ones afterwards)" % args.spares)
        else:
            cfg["fallback"] = ("every instance that fails from its warm guess is solved again from the plain guess; "
                               "those still iterating once at most %g of an m-group is are started early on a "
                               "second thread (same results, shorter wall time)" % args.speculate
                               if args.speculate > 0 else "after the warm solve of each m-group")
    else:
        instances = cs.workloads.vdp_batch(args.batch, seed=SEED + rank)
        cfg = {"workload": "plain batched solve: Van der Pol batch, %d instances (x0~U[-2,2]^2, T~U[2,8], "
                           "r~logU[0.1,10], N~U{32..2048} intervals, m~U{3,4,5}, zero guess, tol 1e-6, seed %d + rank)"
                           % (args.batch, SEED),
               "batch_per_gpu": args.batch, "warm_start": "plain (zero initial guess)", "precision": "fp64",
               "l2": "working set %s GB per step, larger than L2 (129 MB)"}
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, instances, cfg, cores)
        return
    # CPU baseline first: its spawned pool starts before any GPU call
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        _log("CPU baseline (oracle on %d cores)" % cores)
        cpu = _cpu_baseline(instances, cores, family=args.family if args.workload == "warm" else "vdp")
        _log("CPU baseline: %.3g solves/s" % cpu["value"])
    if args.workload == "warm":
        run_warm(args, cs, rank, world, local_rank, cpu, cfg)
    else:
        run_plain(args, cs, rank, world, local_rank, cpu, cfg, instances)


if __name__ == "__main__":
    main()
