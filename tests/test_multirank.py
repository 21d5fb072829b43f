"""bench.py's replica path under several ranks, on the CPU (gloo, world size 2).

The grid step is not sharded (one GB300 runs a whole cell), so N GPUs run N
independent replicas with no data-path collective.  The host logic around
them: the job's time is the slowest rank's (an all-reduce of the maximum),
the rate counts every rank's steps, and the reference arm runs on rank 0
alone, the other ranks leaving without work.
"""
import io
import os
import socket
from contextlib import redirect_stdout

import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [3.0, 5.0, 4.0, 2.0][rank]  # each rank's time per step
        slowest = bench.max_over_ranks(ms, device="cpu")
        q.put((rank, slowest, bench.replica_rate(world, slowest)))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    ps = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [5.0, 5.0]              # every rank sees the slowest rank's time
    assert [g[2] for g in got] == [400.0, 400.0]          # 2 replicas x 1000 / 5 ms steps/s


def test_single_process_keeps_its_value():
    assert bench.max_over_ranks(7.5, device="cpu") == 7.5
    assert bench.replica_rate(1, 4.0) == 250.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    out = io.StringIO()
    with redirect_stdout(out):
        bench.run_reference(None)  # returns before it reads its arguments
    assert out.getvalue() == ""
