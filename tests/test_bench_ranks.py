"""The benchmark's multi-rank aggregation (replicas, no data-path collective): world_size 2 over gloo on
the CPU.  Each rank reports its timed-region seconds; the whole-job value counts every rank's steps over
the slowest rank's time."""
import os

import pytest


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    value, total = bench.aggregate_ranks(torch, dist, world, local_seconds=1.0 + rank, steps=5, device="cpu")
    q.put((rank, value, total))
    dist.destroy_process_group()


def test_aggregate_ranks_gloo_world2():
    import multiprocessing as mp
    import socket
    ctx = mp.get_context("spawn")
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p_ in procs:
        p_.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p_ in procs:
        p_.join(timeout=60)
        assert p_.exitcode == 0
    for rank, value, total in out:
        assert total == pytest.approx(2.0)          # the slower rank's time
        assert value == pytest.approx(2 * 5 / 2.0)  # both ranks' steps over it
