"""The benchmark's multi-rank host logic on CPU: world_size 2 over gloo.

The path does not exchange data between GPUs (independent replicas), so the
only cross-rank steps are the barriers, the max-over-ranks of the timed
region and rank 0 alone printing (and, for --impl reference, rank 0 alone
doing the CPU work)."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 100 * (r + 1) ms for 4 steps of 1000 rays
        total = bench.reduce_max(100.0 * (rank + 1), dist, device="cpu")
        value = bench.whole_job_value(1000, 4, world, total)
        dist.barrier()
        # the reference arm: only rank 0 works and prints
        buf = io.StringIO()
        if rank != 0:
            class A:
                steps, warmup, gpus = 1, 0, world
            with redirect_stdout(buf):
                bench.run_reference(A())
        q.put((rank, total, value, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, total, value, printed = q.get(timeout=120)
        out[rank] = (total, value, printed)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        total, value, _ = out[rank]
        assert total == pytest.approx(200.0)  # max over ranks
        # 2 ranks x 1000 rays x 4 steps in 0.2 s = 0.04 Mrays/s
        assert value == pytest.approx(2 * 1000 * 4 / 0.2 / 1e6)
    assert out[1][2] == ""  # rank 1 runs no reference work and prints nothing


def test_single_rank_is_plain():
    import bench
    assert bench.reduce_max(12.5, None) == 12.5
    assert bench.whole_job_value(8294400, 10, 1, 52.5) == pytest.approx(8294400 * 10 / 0.0525 / 1e6)
