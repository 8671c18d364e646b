"""One batch across several GPUs: contiguous trajectory slices, one per device (or per rank), and
a host gather in trajectory order.  No collective touches the data path.

The reference fans a batch out over its worker threads and collects the per-trajectory results
in index order, reporting the first failing trajectory as ``"trajectory {i}: {msg}"``
(rust/src/lindblad/ode_batch.rs:270-309).  Here the workers are GPUs: a batch is cut into
contiguous slices (equal counts, or balanced by an estimated cost per trajectory for mixed end
times or systems), every slice is solved on its own device through the ordinary batch entry
point, and the slices' values, statistics and first error are put back together exactly as one
call over the whole batch would have returned them.

Two drivers share the cutting and the merging:
* ``solve_batch_across_devices``: one process, one host thread per visible device;
* ``solve_batch_distributed``: one process per GPU (torchrun ranks); every rank solves its slice
  and the slices travel to every rank as Python objects over the process group (the result
  gather on the host, after the solves).
"""

from __future__ import annotations

import re
import threading
from typing import Any, Callable, Sequence

import numpy as np

from .sharding import cost_balanced_bounds

# (lo, hi) -> the batch entry point's 5-tuple (times, flat values, width, time_count, stats) for
# trajectories lo..hi-1 of the batch
SliceSolver = Callable[[int, int], tuple]

_TRAJ_ERR = re.compile(r"^trajectory (\d+): (.*)$", re.S)


def split_batch(n_traj: int, world: int, costs: Sequence[float] | None = None) -> list[tuple[int, int]]:
    """Contiguous [lo, hi) slices, one per worker: equal counts, or balanced by `costs`."""
    if n_traj < 0:
        raise ValueError("n_traj must be non-negative")
    if costs is None:
        costs = np.ones(n_traj)
    if len(costs) != n_traj:
        raise ValueError(f"costs has {len(costs)} entries for {n_traj} trajectories")
    return cost_balanced_bounds(costs, world)


class _SliceFailure:
    """A slice's exception, kept to be raised in trajectory order after every slice is in."""

    __slots__ = ("lo", "exc")

    def __init__(self, lo: int, exc: BaseException) -> None:
        self.lo = lo
        self.exc = exc


def _reraise(failure: _SliceFailure) -> None:
    exc = failure.exc
    m = _TRAJ_ERR.match(str(exc)) if isinstance(exc, ValueError) else None
    if m:
        raise ValueError(f"trajectory {failure.lo + int(m.group(1))}: {m.group(2)}") from exc
    raise exc


def merge_slices(bounds: Sequence[tuple[int, int]], results: Sequence[Any], per_trajectory_times: bool) -> tuple:
    """The batch entry point's 5-tuple for the whole batch from its slices' (in `bounds` order).

    A slice that failed holds a ``_SliceFailure``; the first one in trajectory order is raised,
    with a ``"trajectory {i}: ..."`` message renumbered to the whole batch's index.  Empty slices
    (more workers than trajectories) hold None."""
    for r in results:
        if isinstance(r, _SliceFailure):
            _reraise(r)
    done = [(b, r) for b, r in zip(bounds, results) if r is not None]
    if not done:
        return np.zeros(0), np.zeros(0), 0, 0, {"accepted_steps": 0, "rejected_steps": 0, "rhs_calls": 0,
                                                "event_triggered": False, "event_triggered_by_trajectory": [],
                                                "event_times": [], "event_count": 0}
    widths = {int(r[2]) for _, r in done}
    counts = {int(r[3]) for _, r in done}
    if len(widths) != 1 or len(counts) != 1:
        raise RuntimeError("slices disagree on the output width or point count")
    values = np.concatenate([np.asarray(r[1]).reshape(-1) for _, r in done])
    if per_trajectory_times:
        times = np.concatenate([np.asarray(r[0], dtype=np.float64).reshape(-1) for _, r in done])
    else:
        times = np.asarray(done[0][1][0], dtype=np.float64)
    st0 = done[0][1][4]
    stats: dict[str, Any] = {"solver": st0.get("solver")} if "solver" in st0 else {}
    for key in ("accepted_steps", "rejected_steps", "rhs_calls", "event_count"):
        stats[key] = int(sum(int(r[4].get(key, 0)) for _, r in done))
    stats["event_triggered"] = any(bool(r[4].get("event_triggered", False)) for _, r in done)
    stats["event_triggered_by_trajectory"] = [x for _, r in done for x in r[4].get("event_triggered_by_trajectory", [])]
    stats["event_times"] = [x for _, r in done for x in r[4].get("event_times", [])]
    return times, values, widths.pop(), counts.pop(), stats


def _run_slice(solver: SliceSolver, lo: int, hi: int):
    if hi <= lo:
        return None
    try:
        return solver(lo, hi)
    except Exception as exc:  # kept and raised in trajectory order by merge_slices
        return _SliceFailure(lo, exc)


def solve_batch_distributed(solver: SliceSolver, n_traj: int, *, costs: Sequence[float] | None = None,
                            per_trajectory_times: bool = False, group=None) -> tuple:
    """One slice per rank of the default (or given) process group: this rank solves its slice
    with `solver`, the slices are exchanged as host objects, and every rank returns the whole
    batch's result (or raises its first error)."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    bounds = split_batch(n_traj, world, costs)
    lo, hi = bounds[rank]
    mine = _run_slice(solver, lo, hi)
    if isinstance(mine, _SliceFailure):
        # exceptions travel as (type name, message): enough to raise the same error everywhere
        mine = _SliceFailure(lo, _portable(mine.exc))
    gathered: list[Any] = [None] * world
    dist.all_gather_object(gathered, mine, group=group)
    return merge_slices(bounds, gathered, per_trajectory_times)


def _portable(exc: BaseException) -> BaseException:
    for kind in (ValueError, NotImplementedError, TypeError, RuntimeError):
        if isinstance(exc, kind):
            return kind(str(exc))
    return RuntimeError(f"{type(exc).__name__}: {exc}")


def solve_batch_across_devices(payload: dict, packed_rho0_batch, t0, t1, abstol, reltol, dt, *,
                               devices: Sequence[int] | None = None, costs: Sequence[float] | None = None,
                               parameter_batch=None, **kwargs) -> tuple:
    """``solve_lindblad_batch_ode_py`` over several GPUs of this process: the batch is cut into one
    contiguous slice per device (balanced by `costs` when given), each slice is solved on its own
    device by a plan prepared there, and the results come back in trajectory order.  `kwargs` are
    the batch entry point's keyword arguments (solver, output, parameter_slot_indices, ...)."""
    import torch

    from . import centrex_tlf_rust as api

    if devices is None:
        devices = list(range(torch.cuda.device_count()))
    if not devices:
        raise RuntimeError("no CUDA device is available: the GB300 solver has no CPU fallback")
    rho0 = np.asarray(packed_rho0_batch, dtype=np.float64)
    if rho0.ndim != 2:
        raise ValueError("packed_rho0_batch must be 2D")
    n_traj = rho0.shape[0]
    pb = None if parameter_batch is None else np.asarray(parameter_batch, dtype=np.complex128)
    bounds = split_batch(n_traj, len(devices), costs)
    results: list[Any] = [None] * len(devices)

    def work(k: int) -> None:
        lo, hi = bounds[k]

        def solve(a: int, b: int):
            # a plan per slice: each device holds its own image, and calls on different plans run
            # concurrently (the library serialises calls per plan)
            torch.cuda.set_device(devices[k])
            plan = api.prepare_lindblad_problem_py(payload)
            return api.solve_lindblad_batch_ode_py(plan, rho0[a:b], t0, t1, abstol, reltol, dt,
                                                   parameter_batch=None if pb is None else pb[a:b], **kwargs)

        results[k] = _run_slice(solve, lo, hi)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(devices))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    return merge_slices(bounds, results, kwargs.get("stop_event") is not None)
