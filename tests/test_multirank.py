"""The multi-process path of bench.py on CPU ranks (gloo, world size 2).

One lattice per GPU needs no collective inside a step, so bench.py runs
independent replicas under torchrun and reduces only its timings: the job
time is the slowest rank's and the throughput counts every rank's updates.
These tests drive that reduction over gloo with two CPU ranks.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 1.0 + 0.5 * rank            # rank 1 is the slow one
    slow = bench.max_over_ranks(ms, dist, "cpu")
    q.put((rank, slow, bench.aggregate_mlups(1 << 20, slow, world)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_timing_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [1.5, 1.5]
    # 2 ranks x 2^20 nodes per 1.5 ms
    assert out[0][2] == pytest.approx(2 * (1 << 20) / 1.5e-3 / 1e6)
