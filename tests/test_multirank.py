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
    out[rank] = (mx, sm, allx, bench._rank_device({"CUDA_VISIBLE_DEVICES": "4,5"}, rank, world))
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


def test_rank_device_single_process_keeps_environment():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench._rank_device({"CUDA_VISIBLE_DEVICES": "3"}, 0, 1) == "3"
    assert bench._rank_device({}, 1, 2) == "1"
    assert np.isfinite(bench._max_over_ranks(None, 1.5))
