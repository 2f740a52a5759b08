"""The multi-GPU path of bench.py (instance sharding, weak scaling) on CPU:
two gloo ranks on 127.0.0.1.  Each rank draws its own instances (seed + 100
rank), the timing is the maximum over ranks and the throughput the sum; each
rank is pinned to its own GPU of the visible list before any CUDA call."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench._dist_setup(world, rank)
    cs = bench._pkg()
    insts = cs.workloads.vdp_batch(16, seed=7 + 100 * rank)
    x0 = float(insts[0].x0[0])
    mx = bench._max_over_ranks(d, float(rank + 1))
    sm = bench._sum_over_ranks(d, float(10 * (rank + 1)))
    bench._barrier(d)
    allx = [None] * world
    dist.all_gather_object(allx, x0)
    # a rank-local step on the host: this rank's own small instances solved
    # by the oracle, then the whole-job throughput assembled on rank 0 as the
    # bench does (solves summed over ranks, time the maximum over ranks)
    import json
    import time
    from oracle import collocation_oracle as O
    from conftest import OracleProblem
    P = OracleProblem(cs.workloads.vdp_family_problem())
    mine = cs.workloads.vdp_batch(2, seed=7 + 100 * rank, n_range=(12, 20), m_choices=(4,))
    bench._barrier(d)
    t0 = time.perf_counter()
    solved, nodes = 0, []
    for inst in mine:
        P.theta = inst.theta
        t, y, z, p = inst.guess()
        r = O.solve(P, inst.m, cs.tables.lobatto(inst.m), cs.tables.segment_tables(inst.m), T0=t, Y0=y, Z0=z, P0=p)
        solved += int(r.success)
        nodes.append(int(r.N))
    dt = bench._max_over_ranks(d, time.perf_counter() - t0)
    total = bench._sum_over_ranks(d, float(solved))
    line = None
    if rank == 0:
        line = json.dumps({"metric": "oracle solves/s", "value": total / dt, "unit": "solves/s", "n_gpus": world,
                           "scaling": "weak", "solved": total})
    out[rank] = (mx, sm, allx, bench._rank_device({"CUDA_VISIBLE_DEVICES": "4,5"}, rank, world), solved, nodes, line)
    d.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    world = 2
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    r0, r1 = out[0], out[1]
    assert r0[0] == r1[0] == 2.0          # max over ranks of the step time
    assert r0[1] == r1[1] == 30.0         # sum over ranks of the solves
    assert r0[2][0] != r0[2][1]           # each rank solves its own instances
    assert (r0[3], r1[3]) == ("4", "5")   # one visible GPU per rank
    # the rank-local solves: each rank its own instances, one line from rank 0
    import json
    assert r0[5] != r1[5] or r0[2][0] != r0[2][1]
    assert r1[6] is None
    line = json.loads(r0[6])
    assert line["solved"] == r0[4] + r1[4] == 4 and line["n_gpus"] == 2 and line["value"] > 0


def test_rank_device_single_process_keeps_environment():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench._rank_device({"CUDA_VISIBLE_DEVICES": "3"}, 0, 1) == "3"
    assert bench._rank_device({}, 1, 2) == "1"
    assert np.isfinite(bench._max_over_ranks(None, 1.5))
