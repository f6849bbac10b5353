"""The benchmark's multi-rank paths (no data-path collective), world_size 2 over gloo on the CPU: the
single-domain replicas (each rank reports its timed-region seconds; the whole-job value counts every rank's
steps over the slowest rank's time) and the ensemble split over ranks (each rank solves its share of the
members; converged members are summed over the slowest rank's time)."""
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


def test_shard_members_covers_every_member_once_and_balances():
    """The ensemble split over GPUs (wavi_gb300.ensemble.shard_members): every member on exactly one rank,
    no rank above the average load plus the largest member, the same split on every call."""
    import numpy as np
    from wavi_gb300.ensemble import shard_members
    rng = np.random.default_rng(6)  # the ensemble's own size draw: nx U{64..512} x ny U{16..128}
    costs = rng.integers(64, 513, size=256) * rng.integers(16, 129, size=256)
    for world in (1, 2, 3, 4, 8):
        parts = shard_members(costs, world)
        assert len(parts) == world
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(costs)))
        loads = [float(sum(costs[k] for k in p)) for p in parts]
        assert max(loads) <= sum(loads) / world + max(costs)
        assert parts == shard_members(costs, world)
    with pytest.raises(ValueError):
        shard_members(costs, 0)


def _ensemble_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out = bench.aggregate_ensemble(torch, dist, world, local_seconds=2.0 + rank, local_converged=100 + 20 * rank,
                                   steps=2, device="cpu")
    q.put((rank, *out))
    dist.destroy_process_group()


def test_aggregate_ensemble_gloo_world2():
    """The sharded ensemble's whole-job value: both ranks' converged members over the slower rank's time."""
    import multiprocessing as mp
    import socket
    ctx = mp.get_context("spawn")
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_ensemble_worker, args=(r, 2, port, q)) for r in range(2)]
    for p_ in procs:
        p_.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p_ in procs:
        p_.join(timeout=60)
        assert p_.exitcode == 0
    for rank, value, total, conv in out:
        assert total == pytest.approx(3.0)
        assert conv == 220
        assert value == pytest.approx(220 * 2 / 3.0)
