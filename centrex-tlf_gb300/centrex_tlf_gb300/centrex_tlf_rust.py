"""Drop-in replacement of the reference's native Lindblad entry points.

The reference's Python surface imports four functions from its PyO3 extension
``centrex_tlf.centrex_tlf_rust`` (centrex_tlf/lindblad/plan_static.py:180, solve.py:419,
batch.py:235, batch.py:440).  This module provides the same four names, signatures, defaults,
return tuples and error messages (rust/src/lindblad/python_api.rs:271-799), backed by the
GB300 CUDA solver.  ``install()`` registers it under that import path so the reference's own
``solve_lindblad``/``solve_lindblad_batch``/``parameter_scan``/``initial_condition_scan``/
``grid_scan`` drive the GPU unchanged.

Only ``mode="expanded_sparse"`` runs here (with every solver of the reference: ``dopri5``,
``tsit5``, ``fixed_dopri5``, ``fixed_rk2``, ``fixed_rk4``); the reference's other execution modes
raise ``NotImplementedError``.  The extra keyword ``precision="mixed"`` (adaptive solvers only)
selects single-precision RHS products with double-precision state, error norm and controller.
"""

from __future__ import annotations

import math
import sys
from typing import Any

import numpy as np

from ._options import INTEGRAL_OUTPUTS, RATE_OUTPUTS, SolveOptions
from .native import NativePlan

__all__ = [
    "PreparedLindbladPlan",
    "autotune_lindblad_batch_py",
    "debug_effective_lindblad_rhs_py",
    "prepare_effective_lindblad_plan_py",
    "solve_effective_lindblad_batch_py",
    "solve_effective_lindblad_py",
    "install",
    "prepare_lindblad_problem_py",
    "solve_lindblad_batch_ode_py",
    "solve_lindblad_grid_ode_py",
    "solve_lindblad_multi_batch_ode_py",
    "solve_lindblad_ode_py",
]

_KNOWN_MODES = {
    "reference",
    "structured",
    "structured_upper",
    "expanded_sparse",
    "experimental_expanded_sparse_baseline_packed",
    "experimental_expanded_sparse_current_split_inputs",
    "experimental_expanded_sparse_split_coefficients",
    "experimental_expanded_sparse_split_inputs",
    "experimental_expanded_sparse_precomputed_inputs",
}
_SOLVERS = ("dopri5", "tsit5", "fixed_dopri5", "fixed_rk2", "fixed_rk4")


def _rust_repr(s: str) -> str:
    return '"' + str(s).replace("\\", "\\\\").replace('"', '\\"') + '"'


def _check_mode(mode: str) -> None:
    # ExecutionMode::from_str (rust/src/lindblad/rhs.rs:41-65)
    if mode not in _KNOWN_MODES:
        raise ValueError(f"unsupported execution mode {_rust_repr(mode)}")
    if mode != "expanded_sparse":
        raise NotImplementedError(
            f"execution_mode={mode!r} is not part of the GB300 solver; it implements 'expanded_sparse'"
        )


def _check_solver(solver: str) -> None:
    # OdeSolver::from_str (rust/src/ode/batch.rs:17-29)
    if solver not in _SOLVERS:
        raise ValueError(
            "solver must be 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', or 'fixed_rk4', "
            f"got {_rust_repr(solver)}"
        )


def _time_tol(t: float) -> float:
    return 10.0 * np.finfo(np.float64).eps * max(abs(t), 1.0)


def _fmt(v: float) -> str:
    """Rust's Display for f64 (shortest round-trip, positional)."""
    if math.isnan(v):
        return "NaN"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    r = repr(float(v))
    if "e" not in r and "E" not in r:
        return r[:-2] if r.endswith(".0") else r
    mant, exp = r.lower().split("e")
    exp = int(exp)
    neg = mant.startswith("-")
    mant = mant.lstrip("-")
    digits = mant.replace(".", "")
    point = (mant.index(".") if "." in mant else len(mant)) + exp
    if point <= 0:
        out = "0." + "0" * (-point) + digits
    elif point >= len(digits):
        out = digits + "0" * (point - len(digits))
    else:
        out = digits[:point] + "." + digits[point:]
    out = out.rstrip("0").rstrip(".") if "." in out else out
    return ("-" if neg else "") + out


def _save_plan(saveat: np.ndarray | None, t0: float, t1: float, save_start: bool) -> list[float] | None:
    """build_save_plan (rust/src/ode/common.rs:124-151)."""
    if saveat is None:
        return None
    times: list[float] = []
    if save_start:
        times.append(t0)
    for t in np.asarray(saveat, dtype=np.float64).reshape(-1):
        t = float(t)
        if save_start and abs(t - t0) <= _time_tol(t0):
            continue
        if not math.isfinite(t):
            raise ValueError("saveat contains non-finite value")
        if t < t0 - _time_tol(t0) or t > t1 + _time_tol(t1):
            raise ValueError(f"saveat value {_fmt(t)} is outside [{_fmt(t0)}, {_fmt(t1)}]")
        times.append(t)
    return times


class PreparedLindbladPlan:
    """Opaque prepared plan (the reference's ``PreparedLindbladPlan`` pyclass)."""

    def __init__(self, payload: dict) -> None:
        self.native = NativePlan(payload)

    def n_states(self) -> int:
        return self.native.n_states

    def __repr__(self) -> str:
        return f"PreparedLindbladPlan(n_states={self.native.n_states}, backend='gb300')"


def prepare_lindblad_problem_py(payload: dict) -> PreparedLindbladPlan:
    """rust/src/lindblad/python_api.rs:271-274 -> plan.rs:1155-1308."""
    return PreparedLindbladPlan(payload)


def _native(plan: Any) -> NativePlan:
    if isinstance(plan, PreparedLindbladPlan):
        return plan.native
    if isinstance(plan, NativePlan):
        return plan
    raise TypeError("plan must be a PreparedLindbladPlan from prepare_lindblad_problem_py")


def _output_kind(output: str, output_indices, integral_weights) -> None:
    if output == "selected" and output_indices is None:
        raise ValueError("output='selected' requires output_indices")
    if (output in INTEGRAL_OUTPUTS or output in RATE_OUTPUTS) and integral_weights is None:
        raise ValueError(f"output='{output}' requires integral_weights")


def _opts(native: NativePlan, *, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output,
          output_indices, output_when, integral_weights, stop_event, precision) -> SolveOptions:
    return native.options(
        t0=t0, t1=t1, abstol=abstol, reltol=reltol, dt=dt, saveat=saveat, save_start=save_start,
        maxiters=maxiters, solver=solver, output=output, output_indices=output_indices,
        output_when=output_when, integral_weights=integral_weights, stop_event=stop_event,
        precision=precision,
    )


def solve_lindblad_ode_py(
    plan,
    packed_rho0,
    t0,
    t1,
    abstol,
    reltol,
    dt,
    saveat=None,
    save_start=True,
    maxiters=100000,
    mode="expanded_sparse",
    solver="dopri5",
    output="full",
    output_indices=None,
    output_when="saveat",
    integral_weights=None,
    stop_event=None,
    use_split_input_rhs=True,
    precision="fp64",
):
    """One trajectory (rust/src/lindblad/python_api.rs:422-528).

    Returns ``(times, values, width, stats)``; ``values`` is flat (complex for 'selected').
    ``use_split_input_rhs`` selects a CPU kernel variant in the reference and is accepted for
    compatibility.  ``precision="mixed"`` runs the FP32-RHS / FP64-accumulate form.
    """
    native = _native(plan)
    _check_mode(mode)
    _check_solver(solver)
    _output_kind(output, output_indices, integral_weights)
    kind = output if output in ("populations", "selected") or output in INTEGRAL_OUTPUTS or output in RATE_OUTPUTS else "full"
    rho0 = np.ascontiguousarray(np.asarray(packed_rho0, dtype=np.float64).reshape(-1))
    if rho0.size != native.packed_len:
        raise ValueError(f"expected {native.packed_len}, got {rho0.size}")
    opts = _opts(native, t0=float(t0), t1=float(t1), abstol=abstol, reltol=reltol, dt=dt,
                 saveat=None if saveat is None else np.asarray(saveat, dtype=np.float64), save_start=save_start,
                 maxiters=maxiters, solver=solver, output=kind, output_indices=output_indices,
                 output_when=output_when, integral_weights=integral_weights, stop_event=stop_event,
                 precision=precision)
    times, values, width, st = native.solve_single(opts, rho0)
    stats = {
        "solver": solver,
        "accepted_steps": st["accepted_steps"],
        "rejected_steps": st["rejected_steps"],
        "rhs_calls": st["rhs_calls"],
        "event_triggered": st["event_triggered"],
    }
    if st["event_triggered"]:
        stats["event_time"] = st["event_time"]
        stats["event_index"] = 0
    return np.asarray(times, dtype=np.float64), values, int(width), stats


def _batch_common(native, t0, t1, saveat, save_start, output, output_when, integral_weights, output_indices, stop_event):
    """Option mapping of python_api.rs:589-617 / 723-746 and the point count per trajectory."""
    if output not in ("populations", "selected", "full") and output not in INTEGRAL_OUTPUTS and output not in RATE_OUTPUTS:
        raise ValueError(f"unknown output mode: {_rust_repr(output)}")
    _output_kind(output, output_indices, integral_weights)
    final_integral = output_when == "final" and output in INTEGRAL_OUTPUTS
    saveat_vec = None if saveat is None else np.asarray(saveat, dtype=np.float64).reshape(-1)
    if output_when == "final" and not final_integral:
        saveat_vec = np.array([t1], dtype=np.float64)
    eff_save_start = bool((output_when != "final" or final_integral) and save_start)
    plan_times = _save_plan(saveat_vec, t0, t1, eff_save_start)
    if t1 == t0:
        raise NotImplementedError("a zero-length time span is not supported by the GB300 batch solver")
    if plan_times is not None:
        if output in INTEGRAL_OUTPUTS and output_when != "saveat":
            time_count, ref_times = 1, [plan_times[-1] if plan_times else t1]
        else:
            time_count, ref_times = len(plan_times), list(plan_times)
    elif output in INTEGRAL_OUTPUTS and output_when != "saveat":
        time_count, ref_times = 1, [t1]
    else:
        raise NotImplementedError(
            "batch outputs at every accepted step (saveat=None with output_when='saveat') are not "
            "supported by the GB300 solver; pass explicit saveat values"
        )
    return saveat_vec, eff_save_start, time_count, ref_times


def _batch_result(values, stats_arr, width, time_count, ref_times, t1, solver, stop_event, is_complex):
    triggered = [bool(x) for x in stats_arr["event_triggered"]]
    last_t = ref_times[-1] if ref_times else t1
    event_times = [float(stats_arr["event_time"][i]) if triggered[i] else float(last_t) for i in range(len(triggered))]
    times = np.asarray(event_times if stop_event is not None else ref_times, dtype=np.float64)
    flat = np.ascontiguousarray(values).reshape(-1)
    stats = {
        "solver": solver,
        "accepted_steps": int(stats_arr["accepted_steps"].sum()),
        "rejected_steps": int(stats_arr["rejected_steps"].sum()),
        "rhs_calls": int(stats_arr["rhs_calls"].sum()),
        "event_triggered": any(triggered),
        "event_triggered_by_trajectory": triggered,
        "event_times": event_times,
        "event_count": sum(triggered),
    }
    return times, flat, int(width), int(time_count), stats


def solve_lindblad_batch_ode_py(
    plan,
    packed_rho0_batch,
    t0,
    t1,
    abstol,
    reltol,
    dt,
    saveat=None,
    save_start=True,
    maxiters=100000,
    mode="expanded_sparse",
    solver="dopri5",
    output="populations",
    output_indices=None,
    output_when="final",
    integral_weights=None,
    parameter_slot_indices=None,
    parameter_batch=None,
    parallel=True,
    threads=None,
    stop_event=None,
    use_split_input_rhs=True,
    precision="fp64",
):
    """B trajectories, one GPU launch (rust/src/lindblad/python_api.rs:530-669 ->
    rust/src/lindblad/ode_batch.rs:176-351).  ``parallel``/``threads`` choose the reference's
    CPU thread pool and are accepted for compatibility.

    Returns ``(times, values, width, time_count, stats)``."""
    prep = _prepare_batch(plan, packed_rho0_batch, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, mode,
                          solver, output, output_indices, output_when, integral_weights, parameter_slot_indices,
                          parameter_batch, stop_event, precision)
    if prep.empty is not None:
        return prep.empty
    values, st = prep.native.solve_batch(prep.opts, prep.batch, prep.slots, prep.pv, prep.time_count)
    return prep.result(values, st)


class _PreparedBatch:
    """A validated batch: the native plan, options, inputs and the result shaping of one call."""

    __slots__ = ("native", "batch", "slots", "pv", "opts", "time_count", "ref_times", "t1", "solver", "stop_event", "empty")

    def result(self, values, st):
        return _batch_result(values, st, self.opts.width, self.time_count, self.ref_times, self.t1, self.solver,
                             self.stop_event, self.opts.is_complex)


def _prepare_batch(plan, packed_rho0_batch, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, mode, solver,
                   output, output_indices, output_when, integral_weights, parameter_slot_indices, parameter_batch,
                   stop_event, precision) -> _PreparedBatch:
    native = _native(plan)
    _check_mode(mode)
    _check_solver(solver)
    batch = np.asarray(packed_rho0_batch, dtype=np.float64)
    if batch.ndim != 2:
        raise ValueError("packed_rho0_batch must be 2D")
    if batch.shape[1] != native.packed_len:
        raise ValueError(f"rho0 dim mismatch: {batch.shape[1]} vs {native.packed_len}")
    t0, t1 = float(t0), float(t1)
    slots = list(parameter_slot_indices or [])
    if parameter_batch is not None:
        pv = np.asarray(parameter_batch, dtype=np.complex128)
        if pv.ndim != 2 or pv.shape[0] != batch.shape[0] or pv.shape[1] != len(slots):
            raise ValueError("parameter_batch shape mismatch")
    else:
        pv = None
    prep = _PreparedBatch()
    prep.native, prep.batch, prep.t1, prep.solver, prep.stop_event = native, batch, t1, solver, stop_event
    prep.empty = None
    if batch.shape[0] == 0:
        prep.empty = (np.zeros(0), np.zeros(0), 0, 0, {
            "solver": solver, "accepted_steps": 0, "rejected_steps": 0, "rhs_calls": 0, "event_triggered": False,
            "event_triggered_by_trajectory": [], "event_times": [], "event_count": 0})
        return prep
    saveat_vec, eff_ss, time_count, ref_times = _batch_common(
        native, t0, t1, saveat, save_start, output, output_when, integral_weights, output_indices, stop_event
    )
    prep.opts = _opts(native, t0=t0, t1=t1, abstol=abstol, reltol=reltol, dt=dt, saveat=saveat_vec, save_start=eff_ss,
                      maxiters=maxiters, solver=solver, output=output, output_indices=output_indices,
                      output_when=output_when, integral_weights=integral_weights, stop_event=stop_event,
                      precision=precision)
    use = pv is not None and len(slots) > 0
    prep.slots, prep.pv = (slots, pv) if use else (None, None)
    prep.time_count, prep.ref_times = time_count, ref_times
    return prep


_BATCH_DEFAULTS = dict(saveat=None, save_start=True, maxiters=100000, mode="expanded_sparse", solver="dopri5",
                       output="populations", output_indices=None, output_when="final", integral_weights=None,
                       parameter_slot_indices=None, parameter_batch=None, stop_event=None, precision="fp64")


def solve_lindblad_multi_batch_ode_py(jobs, precision=None):
    """Several batches on different plans (systems of different sizes) in one GPU call
    (obe_solve_multi_device).  The reference has no counterpart: it solves one prepared plan per
    call (rust/src/lindblad/ode_batch.rs:176-351), so a mixed workload there is one call per plan.

    ``jobs`` is a sequence of dicts, each holding the arguments of ``solve_lindblad_batch_ode_py``
    by name (``plan``, ``packed_rho0_batch``, ``t0``, ``t1``, ``abstol``, ``reltol``, ``dt`` and any
    of its keywords).  ``precision``, when given, applies to every job.  The jobs' kernels run
    concurrently on the GPU, the largest systems first.  Returns one
    ``(times, values, width, time_count, stats)`` per job, as ``solve_lindblad_batch_ode_py``
    would; a failing trajectory raises ``ValueError("job {k}: trajectory {i}: {msg}")``."""
    import torch

    from .native import multi_solve_device

    preps = []
    for k, job in enumerate(jobs):
        kw = dict(_BATCH_DEFAULTS)
        unknown = set(job) - set(kw) - {"plan", "packed_rho0_batch", "t0", "t1", "abstol", "reltol", "dt",
                                         "parallel", "threads", "use_split_input_rhs"}
        if unknown:
            raise TypeError(f"job {k}: unexpected arguments {sorted(unknown)}")
        kw.update({key: v for key, v in job.items() if key in kw})
        if precision is not None:
            kw["precision"] = precision
        try:
            preps.append(_prepare_batch(job["plan"], job["packed_rho0_batch"], job["t0"], job["t1"], job["abstol"],
                                        job["reltol"], job["dt"], kw["saveat"], kw["save_start"], kw["maxiters"],
                                        kw["mode"], kw["solver"], kw["output"], kw["output_indices"],
                                        kw["output_when"], kw["integral_weights"], kw["parameter_slot_indices"],
                                        kw["parameter_batch"], kw["stop_event"], kw["precision"]))
        except (ValueError, NotImplementedError, TypeError) as exc:
            raise type(exc)(f"job {k}: {exc}") from None
    live = [k for k, p in enumerate(preps) if p.empty is None]
    dev = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else None
    if live and dev is None:
        raise RuntimeError("no CUDA device is available: the GB300 solver has no CPU fallback")
    bufs = {}
    for k in live:
        p = preps[k]
        b = p.batch.shape[0]
        vals = p.time_count * p.opts.width * (2 if p.opts.is_complex else 1)
        bufs[k] = {
            "rho0": torch.from_numpy(np.ascontiguousarray(p.batch)).to(dev),
            "params": (torch.from_numpy(np.ascontiguousarray(p.pv).view(np.float64)).to(dev)
                       if p.pv is not None else None),
            "values": torch.empty(b * vals, dtype=torch.float64, device=dev),
            "stats": torch.zeros(b * 6, dtype=torch.int64, device=dev),
        }
    if live:
        stream = torch.cuda.current_stream(dev)
        multi_solve_device(
            [(preps[k].native, preps[k].opts, preps[k].batch.shape[0], bufs[k]["rho0"].data_ptr(), preps[k].slots,
              bufs[k]["params"].data_ptr() if bufs[k]["params"] is not None else None, preps[k].time_count,
              bufs[k]["values"].data_ptr(), bufs[k]["stats"].data_ptr()) for k in live],
            stream.cuda_stream)
        stream.synchronize()
    out = []
    for k, p in enumerate(preps):
        if p.empty is not None:
            out.append(p.empty)
            continue
        from . import _abi

        st = bufs[k]["stats"].cpu().numpy().view(_abi.TRAJ_STATS_DTYPE)
        if np.any(st["status"] != 0):
            # the device form reports status codes only: re-run this job through the host-pointer
            # call, which fails on the same trajectory with the reference's message
            try:
                p.native.solve_batch(p.opts, p.batch, p.slots, p.pv, p.time_count)
            except ValueError as exc:
                raise ValueError(f"job {k}: {exc}") from None
            raise RuntimeError(f"job {k}: a trajectory failed on the device but not on the re-run")
        values = bufs[k]["values"].cpu().numpy()
        if p.opts.is_complex:
            values = values.view(np.complex128)
        out.append(p.result(values.reshape(p.batch.shape[0], p.time_count, p.opts.width), st))
    return out


def autotune_lindblad_batch_py(plan, packed_rho0_batch, t0, t1, abstol, reltol, dt, probe_steps=64, **kwargs):
    """Choose the GPU launch shape of ``plan`` for batches like this one (obe_plan_autotune): the
    arguments are those of ``solve_lindblad_batch_ode_py``; every candidate shape solves the batch
    with at most ``probe_steps`` steps per trajectory and the fastest is kept for the plan's later
    solves.  No counterpart in the reference (its CPU path has no launch shape).  Returns the
    candidates with their probe times, the chosen one first."""
    import torch

    kw = dict(_BATCH_DEFAULTS)
    unknown = set(kwargs) - set(kw) - {"parallel", "threads", "use_split_input_rhs"}
    if unknown:
        raise TypeError(f"unexpected arguments {sorted(unknown)}")
    kw.update({key: v for key, v in kwargs.items() if key in kw})
    prep = _prepare_batch(plan, packed_rho0_batch, t0, t1, abstol, reltol, dt, kw["saveat"], kw["save_start"],
                          kw["maxiters"], kw["mode"], kw["solver"], kw["output"], kw["output_indices"], kw["output_when"],
                          kw["integral_weights"], kw["parameter_slot_indices"], kw["parameter_batch"], kw["stop_event"],
                          kw["precision"])
    if prep.empty is not None:
        raise ValueError("autotuning needs a non-empty batch")
    if not torch.cuda.is_available():
        raise RuntimeError("no CUDA device is available: the GB300 solver has no CPU fallback")
    dev = torch.device("cuda", torch.cuda.current_device())
    rho0 = torch.from_numpy(np.ascontiguousarray(prep.batch)).to(dev)
    params = (torch.from_numpy(np.ascontiguousarray(prep.pv).view(np.float64)).to(dev) if prep.pv is not None else None)
    stream = torch.cuda.current_stream(dev)
    return prep.native.autotune(prep.opts, prep.batch.shape[0], rho0.data_ptr(), prep.slots,
                                params.data_ptr() if params is not None else None, prep.time_count,
                                probe_steps=probe_steps, stream=stream.cuda_stream)


def solve_lindblad_grid_ode_py(
    plan,
    packed_rho0,
    t0,
    t1,
    abstol,
    reltol,
    dt,
    parameter_slot_indices,
    parameter_axes,
    parameter_axis_lengths,
    saveat=None,
    save_start=True,
    maxiters=100000,
    mode="expanded_sparse",
    solver="dopri5",
    output="populations",
    output_indices=None,
    output_when="final",
    integral_weights=None,
    parallel=True,
    threads=None,
    stop_event=None,
    use_split_input_rhs=True,
    precision="fp64",
):
    """A row-major parameter grid from one rho0 (rust/src/lindblad/python_api.rs:671-799 ->
    rust/src/lindblad/ode_batch.rs:571-1040); last axis fastest."""
    native = _native(plan)
    _check_mode(mode)
    _check_solver(solver)
    lengths = [int(x) for x in parameter_axis_lengths]
    if not lengths:
        raise ValueError("parameter grid must contain at least one axis")
    if any(x == 0 for x in lengths):
        raise ValueError("parameter grid axes must be non-empty")
    rho0 = np.asarray(packed_rho0, dtype=np.float64).reshape(-1)
    t0, t1 = float(t0), float(t1)
    axes_flat = np.asarray(parameter_axes, dtype=np.complex128).reshape(-1)
    axes = []
    off = 0
    for n in lengths:
        axes.append(axes_flat[off: off + n])
        off += n
    saveat_vec, eff_ss, time_count, ref_times = _batch_common(
        native, t0, t1, saveat, save_start, output, output_when, integral_weights, output_indices, stop_event
    )
    opts = _opts(native, t0=t0, t1=t1, abstol=abstol, reltol=reltol, dt=dt, saveat=saveat_vec, save_start=eff_ss,
                 maxiters=maxiters, solver=solver, output=output, output_indices=output_indices,
                 output_when=output_when, integral_weights=integral_weights, stop_event=stop_event,
                 precision=precision)
    values, st = native.solve_grid(opts, rho0, list(parameter_slot_indices), axes, time_count)
    return _batch_result(values, st, opts.width, time_count, ref_times, t1, solver, stop_event, opts.is_complex)


# ---- interpolated effective-Hamiltonian Lindblad path (rust/src/effective_lindblad) --------------


class PreparedEffectiveLindbladPlan:
    """The GB300 counterpart of the reference's EffectiveLindbladPlan pyclass
    (effective_lindblad/plan.rs:43-86): read-only n_states, real_dim, n_grid, slot_names."""

    def __init__(self, plan_dict: dict) -> None:
        self.native = NativePlan.from_effective(plan_dict)
        self.n_states = self.native.n_states
        self.real_dim = self.native.packed_len
        self.n_grid = self.native.arrays.n_grid

    @property
    def slot_names(self) -> list[str]:
        return list(self.native.slot_names)

    def __repr__(self) -> str:
        return f"EffectiveLindbladPlan(n_states={self.n_states}, real_dim={self.real_dim}, n_grid={self.n_grid})"


def prepare_effective_lindblad_plan_py(plan_dict: dict) -> PreparedEffectiveLindbladPlan:
    """effective_lindblad/python_api.rs:16-29."""
    return PreparedEffectiveLindbladPlan(plan_dict)


def _effective_native(plan) -> NativePlan:
    if isinstance(plan, PreparedEffectiveLindbladPlan):
        return plan.native
    raise TypeError("plan must be an EffectiveLindbladPlan from prepare_effective_lindblad_plan_py")


def _effective_output(output: str) -> str:
    # effective_lindblad/solver.rs:102-132: anything but these three kinds is the full state
    if output in ("populations", "selected") or output in INTEGRAL_OUTPUTS:
        return output
    return "full"


def _effective_opts(native, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output, output_indices,
                    integral_weights):
    _check_solver(solver)
    out = _effective_output(output)
    if out == "selected" and output_indices is None:
        raise ValueError("output='selected' requires output_indices")
    if out in INTEGRAL_OUTPUTS and integral_weights is None:
        raise ValueError(f"output='{output}' requires integral_weights")
    sv = None if saveat is None else np.asarray(saveat, dtype=np.float64).reshape(-1)
    # the integral outputs report their final value (WeightedIntegralOutput::finish)
    opts = native.options(t0=float(t0), t1=float(t1), abstol=abstol, reltol=reltol, dt=dt, saveat=sv,
                          save_start=bool(save_start), maxiters=int(maxiters), solver=solver, output=out,
                          output_indices=output_indices, output_when="final", integral_weights=integral_weights,
                          stop_event=None)
    return opts, out, sv


def solve_effective_lindblad_py(plan, y0, t0, t1, abstol, reltol, dt, saveat=None, save_start=True, maxiters=100000,
                                solver="dopri5", output="full", output_indices=None, integral_weights=None):
    """effective_lindblad/python_api.rs:44-92 -> solver.rs:78-132: one trajectory of the split-real
    state; returns ``(times, values, width)`` (values complex for ``selected``)."""
    native = _effective_native(plan)
    y = np.ascontiguousarray(np.asarray(y0, dtype=np.float64).reshape(-1))
    if y.size != native.packed_len:
        raise ValueError(f"expected state length {native.packed_len}, got {y.size}")
    opts, out, _ = _effective_opts(native, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output,
                                   output_indices, integral_weights)
    times, values, width, _ = native.solve_single(opts, y)
    return np.asarray(times, dtype=np.float64), np.ascontiguousarray(values).reshape(-1), int(width)


def solve_effective_lindblad_batch_py(plan, packed_rho0, t0, t1, abstol, reltol, dt, saveat=None, save_start=True,
                                      maxiters=100000, solver="dopri5", output="populations", output_indices=None,
                                      integral_weights=None, parameter_slot_indices=None, parameter_batch=None,
                                      trajectory_count=1, parallel=True, threads=None):
    """effective_lindblad/python_api.rs:154-250 -> solver.rs:134-281: `trajectory_count` solves
    from one initial state with real per-trajectory base-slot values, one GPU launch.  Returns
    ``(times, values, width, time_count, stats)``; selected values interleave (re, im) as the
    reference flattens them.  ``parallel``/``threads`` choose the reference's CPU pool."""
    native = _effective_native(plan)
    y = np.ascontiguousarray(np.asarray(packed_rho0, dtype=np.float64).reshape(-1))
    dim = native.packed_len
    slots = list(parameter_slot_indices or [])
    b = int(trajectory_count)
    if parameter_batch is not None:
        pb = np.asarray(parameter_batch, dtype=np.float64)
        if pb.ndim != 2 or pb.shape[0] != b or pb.shape[1] != len(slots):
            shape = pb.shape if pb.ndim == 2 else (pb.size, 1)
            raise ValueError(f"parameter_batch shape ({shape[0]},{shape[1]}) doesn't match ({b},{len(slots)})")
    else:
        pb = np.zeros((b, len(slots)))
    if y.size != dim:
        raise ValueError(f"expected state length {dim}, got {y.size}")
    opts, out, sv = _effective_opts(native, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output,
                                    output_indices, integral_weights)
    plan_times = _save_plan(sv, float(t0), float(t1), bool(save_start))
    if out in INTEGRAL_OUTPUTS:
        time_count, ref_times = 1, [plan_times[-1] if plan_times else float(t1)]
    elif plan_times is not None:
        time_count, ref_times = len(plan_times), list(plan_times)
    else:
        raise NotImplementedError("batch outputs at every accepted step (saveat=None) are not supported by the GB300 "
                                  "solver; pass explicit saveat values")
    stats = {"solver": solver, "accepted_steps": 0, "rejected_steps": 0, "rhs_calls": 0, "trajectory_count": b}
    if b == 0:
        return np.zeros(0), np.zeros(0), 0, 0, stats
    batch = np.ascontiguousarray(np.broadcast_to(y, (b, dim)))
    use = len(slots) > 0
    values, st = native.solve_batch(opts, batch, slots if use else None, pb.astype(np.complex128) if use else None, time_count)
    stats.update(accepted_steps=int(st["accepted_steps"].sum()), rejected_steps=int(st["rejected_steps"].sum()),
                 rhs_calls=int(st["rhs_calls"].sum()))
    flat = np.ascontiguousarray(values).reshape(-1)
    if opts.is_complex:
        flat = flat.view(np.float64)
    return np.asarray(ref_times, dtype=np.float64), flat, int(opts.width), int(time_count), stats


def debug_effective_lindblad_rhs_py(plan, y0, t):
    """effective_lindblad/python_api.rs:94-152: one RHS and what it read."""
    native = _effective_native(plan)
    dy, info = native.effective_rhs_debug(np.asarray(y0, dtype=np.float64).reshape(-1), float(t))
    return {
        "field_val": float(info[0]), "rabi_val": float(info[1]), "detuning_val": float(info[2]),
        "dy_norm": float(np.sqrt(np.sum(dy * dy))), "dy_max": float(np.max(np.abs(dy))) if dy.size else 0.0,
        "has_nan": bool(np.isnan(dy).any()), "has_inf": bool(np.isinf(dy).any()),
        "last_interval": int(info[3]), "dy": dy,
    }


def install() -> None:
    """Register this module as ``centrex_tlf.centrex_tlf_rust`` so the reference's Python
    surface calls the GB300 solver.  The builder helpers of the reference's extension are
    absent on purpose: the reference falls back to its Python builders
    (centrex_tlf/hamiltonian/generate_hamiltonian.py:18-30)."""
    sys.modules["centrex_tlf.centrex_tlf_rust"] = sys.modules[__name__]
