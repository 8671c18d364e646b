"""One batch over several GPUs, host logic on CPU: the slices' values, statistics and first error
gathered in trajectory order equal a one-worker run (ode_batch.rs:270-309 collects its workers'
results the same way), with two gloo ranks standing in for two GPUs and a stub per-slice solver
(a deterministic function of the global trajectory index) standing in for the device solve."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from centrex_tlf_gb300.multigpu import merge_slices, solve_batch_distributed, split_batch

WIDTH, TC = 3, 2


def stub_solver(fail_at=None, events=False):
    """The batch entry point's 5-tuple for trajectories lo..hi-1, as the GPU would return them."""

    def solve(lo: int, hi: int):
        idx = np.arange(lo, hi)
        if fail_at is not None and lo <= fail_at < hi:
            raise ValueError(f"trajectory {fail_at - lo}: Stopped at x=0.5. Need more than 7 steps.")
        values = (idx[:, None, None] * 100.0 + np.arange(TC)[None, :, None] * 10.0 + np.arange(WIDTH)[None, None, :]).reshape(-1)
        trig = [bool(i % 3 == 0) for i in idx] if events else [False] * idx.size
        ev_t = [0.1 * i if t else 1.0 for i, t in zip(idx, trig)]
        stats = {"solver": "tsit5", "accepted_steps": int((idx + 10).sum()), "rejected_steps": int((idx % 2).sum()),
                 "rhs_calls": int(6 * (idx + 10).sum() + idx.size), "event_triggered": any(trig),
                 "event_triggered_by_trajectory": trig, "event_times": ev_t, "event_count": sum(trig)}
        times = np.asarray(ev_t) if events else np.array([0.5, 1.0])
        return times, values, WIDTH, TC, stats

    return solve


def _merged(n, world, solver, events=False, costs=None):
    bounds = split_batch(n, world, costs)
    results = []
    from centrex_tlf_gb300.multigpu import _run_slice

    for lo, hi in bounds:
        results.append(_run_slice(solver, lo, hi))
    return merge_slices(bounds, results, events)


def _assert_same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2:4] == b[2:4]
    assert a[4] == b[4]


@pytest.mark.parametrize("events", [False, True])
def test_slices_gather_to_the_one_worker_result(events):
    n = 23
    one = _merged(n, 1, stub_solver(events=events), events)
    for world in (2, 3, 5, 40):
        _assert_same(_merged(n, world, stub_solver(events=events), events), one)
    # cost-balanced slices (uneven end times) gather the same way
    costs = np.linspace(1.0, 9.0, n)
    _assert_same(_merged(n, 4, stub_solver(events=events), events, costs=costs), one)


def test_first_error_is_renumbered_to_the_whole_batch():
    with pytest.raises(ValueError) as one:
        _merged(23, 1, stub_solver(fail_at=13))
    for world in (2, 4, 7):
        with pytest.raises(ValueError) as many:
            _merged(23, world, stub_solver(fail_at=13))
        assert str(many.value) == str(one.value) == "trajectory 13: Stopped at x=0.5. Need more than 7 steps."


def test_split_batch_validation():
    assert split_batch(5, 2) == [(0, 2), (2, 5)] or split_batch(5, 2) == [(0, 3), (3, 5)]
    with pytest.raises(ValueError):
        split_batch(3, 2, costs=[1.0, 2.0])


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, n: int, fail_at, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = solve_batch_distributed(stub_solver(fail_at=fail_at, events=True), n, per_trajectory_times=True)
        out.put((rank, "ok", [np.asarray(res[0]).tolist(), np.asarray(res[1]).tolist(), res[2], res[3], res[4]]))
    except ValueError as exc:
        out.put((rank, "error", str(exc)))
    finally:
        dist.destroy_process_group()


def _run_ranks(n, fail_at):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, n, fail_at, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=120) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


def test_two_gloo_ranks_gather_the_batch():
    n = 17
    one = _merged(n, 1, stub_solver(events=True), True)
    for rank, kind, res in _run_ranks(n, None):
        assert kind == "ok"
        np.testing.assert_array_equal(res[0], one[0])
        np.testing.assert_array_equal(res[1], one[1])
        assert (res[2], res[3]) == one[2:4]
        assert res[4] == one[4]


def test_two_gloo_ranks_raise_the_first_error():
    for rank, kind, msg in _run_ranks(17, 12):
        assert kind == "error"
        assert msg == "trajectory 12: Stopped at x=0.5. Need more than 7 steps."
