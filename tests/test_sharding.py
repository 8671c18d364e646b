"""The multi-GPU path's host logic on CPU ranks (gloo, world size 2): disjoint shards that cover
the batch, cost-balanced splits of a mixed batch, and the maximum of the ranks' times."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from centrex_tlf_gb300.sharding import cost_balanced_bounds, max_over_ranks, shard_bounds, trajectory_cost


def test_weak_scaling_shards_partition_the_scan():
    per, world = 4096, 4
    ranges = [shard_bounds(per, r) for r in range(world)]
    covered = np.concatenate([np.arange(lo, hi) for lo, hi in ranges])
    np.testing.assert_array_equal(covered, np.arange(per * world))


def test_cost_balanced_split_of_a_mixed_batch():
    rng = np.random.default_rng(0)
    # 16/39/76-state instances 6:3:1 with end times U[50, 300] (the heterogeneous batch's mix)
    n = rng.choice([16, 39, 76], size=2000, p=[0.6, 0.3, 0.1])
    costs = [trajectory_cost(k * k, t) for k, t in zip(n, rng.uniform(50.0, 300.0, n.size))]
    for world in (1, 2, 3, 8):
        b = cost_balanced_bounds(costs, world)
        assert b[0][0] == 0 and b[-1][1] == len(costs)
        assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
        per = [sum(costs[lo:hi]) for lo, hi in b]
        assert max(per) - min(per) <= max(costs) + 1e-9  # within one trajectory of even
    assert cost_balanced_bounds([0.0, 0.0, 0.0, 0.0], 2) == [(0, 2), (2, 4)]
    with pytest.raises(ValueError):
        cost_balanced_bounds([1.0, -1.0], 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = shard_bounds(10, rank)
    # each rank "times" its shard; the job's time is the slowest rank's
    t = max_over_ranks([1.0 + rank, 5.0 - rank])
    dist.barrier()
    out.put((rank, lo, hi, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_time_the_job_by_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r, lo, hi) for r, lo, hi, _ in res] == [(0, 0, 10), (1, 10, 20)]
    assert all(t == [2.0, 5.0] for *_, t in res)
    # without a process group the values pass through
    assert max_over_ranks([3.0]) == [3.0]
