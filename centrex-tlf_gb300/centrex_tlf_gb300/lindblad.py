"""The reference's Lindblad solve/scan surface over the GB300 solver.

Mirrors ``solve_lindblad`` (centrex_tlf/lindblad/solve.py:504-694, its Rust-native branch
:397-501), ``solve_lindblad_batch``, ``initial_condition_scan``, ``parameter_scan`` and
``grid_scan`` (centrex_tlf/lindblad/batch.py:143-519): same argument names, defaults, validation
messages, option mapping and result shapes.  A problem is prepared from the plan payload the
reference's builders produce (``PreparedLindbladProblem.to_payload()``), so this module runs
without the reference's builders; with them, ``centrex_tlf_rust.install()`` lets the reference's
own surface drive the same solver.
"""

from __future__ import annotations

import time
from collections.abc import Mapping, Sequence
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import numpy.typing as npt

from . import centrex_tlf_rust as native_api
from ._options import INTEGRAL_OUTPUTS, RATE_OUTPUTS

__all__ = [
    "LindbladBatchResult",
    "LindbladObservableResult",
    "LindbladResult",
    "PackedHermitianLayout",
    "PreparedProblem",
    "grid_scan",
    "initial_condition_scan",
    "parameter_scan",
    "population",
    "prepare_from_payload",
    "solve_lindblad",
    "solve_lindblad_batch",
]

WEIGHTED_OUTPUTS = set(INTEGRAL_OUTPUTS) | set(RATE_OUTPUTS)


@dataclass(frozen=True)
class PackedHermitianLayout:
    """Packed Hermitian state layout (centrex_tlf/lindblad/state_layout.py:12-79): the n
    diagonal entries first, then (Re, Im) of the strict upper triangle row by row."""

    n: int

    def __post_init__(self) -> None:
        if self.n <= 0:
            raise ValueError("layout dimension must be positive")

    @property
    def packed_len(self) -> int:
        return self.n * self.n

    def _iu(self):
        return np.triu_indices(self.n, 1)

    def pack(self, matrix) -> np.ndarray:
        arr = np.asarray(matrix, dtype=np.complex128)
        if arr.shape != (self.n, self.n):
            raise ValueError(f"expected matrix shape {(self.n, self.n)}, got {arr.shape}")
        iu = self._iu()
        upper = arr[iu]
        out = np.empty(self.packed_len, dtype=np.float64)
        out[: self.n] = np.real(np.diag(arr))
        out[self.n:: 2] = upper.real
        out[self.n + 1:: 2] = upper.imag
        return out

    def unpack(self, packed) -> np.ndarray:
        arr = np.asarray(packed, dtype=np.float64)
        if arr.shape != (self.packed_len,):
            raise ValueError(f"expected packed vector length {self.packed_len}, got {arr.shape}")
        m = np.zeros((self.n, self.n), dtype=np.complex128)
        m[np.diag_indices(self.n)] = arr[: self.n]
        iu = self._iu()
        vals = arr[self.n:: 2] + 1j * arr[self.n + 1:: 2]
        m[iu] = vals
        m[(iu[1], iu[0])] = np.conjugate(vals)
        return m


@dataclass
class PreparedProblem:
    """What a solve needs from ``PreparedLindbladProblem`` (plan_static.py:21-68)."""

    payload: dict
    layout: PackedHermitianLayout
    parameter_graph: dict
    hamiltonian_plan: dict
    expanded_rhs_plan: dict | None
    rust_plan: Any

    def check_execution_mode(self, execution_mode: str) -> None:
        if "expanded_sparse" not in execution_mode:
            return
        if self.expanded_rhs_plan is not None:
            return
        kind = self.hamiltonian_plan.get("kind", "entrywise")
        raise ValueError(
            f"execution_mode={execution_mode!r} requires a decomposed Hamiltonian "
            f"plan, but this problem was prepared with kind={kind!r}. Either pass "
            "hamiltonian_representation='decomposed' to prepare_lindblad_problem, "
            "or use execution_mode='structured'."
        )


def prepare_from_payload(payload: dict) -> PreparedProblem:
    return PreparedProblem(
        payload=payload,
        layout=PackedHermitianLayout(int(payload["n_states"])),
        parameter_graph=payload["parameter_graph"],
        hamiltonian_plan=payload["hamiltonian_plan"],
        expanded_rhs_plan=payload.get("expanded_rhs_plan"),
        rust_plan=native_api.prepare_lindblad_problem_py(payload),
    )


@dataclass(frozen=True)
class PopulationEvent:
    indices: tuple[int, ...]
    threshold: float = 0.0
    name: str = "population"


def population(index_or_indices, *, threshold: float = 0.0, name: str | None = None) -> PopulationEvent:
    """centrex_tlf/lindblad/events.py:27-40."""
    if isinstance(index_or_indices, (int, np.integer)):
        indices = (int(index_or_indices),)
    else:
        indices = tuple(int(i) for i in index_or_indices)
    if not indices:
        raise ValueError("population event requires at least one index")
    return PopulationEvent(indices=indices, threshold=float(threshold), name=name or "population")


def normalize_stop_event(stop_event, prepared: PreparedProblem) -> dict | None:
    """centrex_tlf/lindblad/events.py:53-94 for the event forms that need no sympy: a
    ``PopulationEvent`` or an already-compiled ``{"kind": ..., ...}`` dict."""
    if stop_event is None:
        return None
    n = prepared.layout.n
    if isinstance(stop_event, PopulationEvent):
        for index in stop_event.indices:
            if index < 0 or index >= n:
                raise ValueError(f"population event index {index} out of bounds for {n} states")
        return {"kind": "population", "indices": list(stop_event.indices), "threshold": stop_event.threshold,
                "name": stop_event.name}
    if isinstance(stop_event, dict) and stop_event.get("kind") in ("population", "runtime_expression"):
        return stop_event
    raise TypeError(
        "stop_event must be a RuntimeExpression, sympy expression, Parameter, PopulationEvent, or None"
    )


@dataclass
class LindbladResult:
    t: npt.NDArray[np.float64]
    packed_y: npt.NDArray[np.float64]
    layout: Any
    solver_stats: dict[str, Any] | None = None

    def density_matrices(self) -> np.ndarray:
        return np.stack([self.layout.unpack(s) for s in self.packed_y]) if len(self.packed_y) else np.zeros((0, self.layout.n, self.layout.n), complex)

    def populations(self) -> np.ndarray:
        return np.asarray(self.packed_y)[:, : self.layout.n]


@dataclass
class LindbladObservableResult:
    t: npt.NDArray[np.float64]
    values: npt.NDArray[Any]
    output: str
    output_indices: Any | None = None
    solver_stats: dict[str, Any] | None = None


@dataclass
class LindbladBatchResult:
    t: npt.NDArray[np.float64]
    values: npt.NDArray[Any]
    output: str
    output_indices: list[tuple[int, int]] | None
    trajectory_count: int
    parameter_slots: list[str] | None = None
    parameter_values: npt.NDArray[np.complex128] | None = None
    solver_stats: dict[str, Any] | None = None
    metadata: dict[str, Any] = field(default_factory=dict)


def _normalize_saveat(saveat, t_span, save_start):
    """solve.py:74-90 / batch.py:47-62."""
    if saveat is None:
        return None
    if isinstance(saveat, (float, int, np.floating, np.integer)):
        step = float(saveat)
        if step <= 0:
            raise ValueError("saveat step must be positive")
        values = np.arange(t_span[0], t_span[1] + 0.5 * step, step, dtype=np.float64)
    else:
        values = np.asarray(saveat, dtype=np.float64)
    if not save_start and values.size > 0 and np.isclose(values[0], t_span[0]):
        values = values[1:]
    return values


def _stats(solver_stats, *, solver, saved_points, elapsed):
    stats = dict(solver_stats)
    stats["solver"] = solver
    stats.setdefault("function_evaluations", stats.get("rhs_calls", 0))
    stats.setdefault("saved_points", saved_points)
    stats.setdefault("rhs_seconds", elapsed)
    stats.setdefault("total_seconds", elapsed)
    return stats


def solve_lindblad(
    prepared: PreparedProblem,
    rho0,
    t_span: Sequence[float],
    *,
    solver: str = "dopri5",
    abstol: float = 1e-7,
    reltol: float = 1e-4,
    dt: float = 1e-8,
    saveat=None,
    save_start: bool = True,
    maxiters: int = 100_000,
    execution_mode: str = "expanded_sparse",
    use_split_input_rhs: bool = True,
    collect_stats: bool = False,
    output: str = "full",
    output_indices=None,
    output_when: str = "saveat",
    dense_output: bool = True,
    integral_weights=None,
    stop_event=None,
    precision: str = "fp64",
):
    """solve.py:504-694, native branch (:397-501)."""
    if solver not in {"dopri5", "tsit5", "fixed_dopri5", "fixed_rk2", "fixed_rk4"}:
        raise NotImplementedError("supported solvers are 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', and 'fixed_rk4'")
    if execution_mode not in {"reference", "structured", "structured_upper", "expanded_sparse"}:
        raise NotImplementedError(
            "supported execution_mode values are 'reference', 'structured', 'structured_upper', and 'expanded_sparse'"
        )
    if output not in {"full", "populations", "selected", *WEIGHTED_OUTPUTS}:
        raise NotImplementedError(
            "output must be 'full', 'populations', 'selected', 'weighted_integral', "
            "'photon_integral', 'excited_population', 'weighted_rate', 'photon_rate', "
            "or 'excited_population_rate'"
        )
    if output_when not in {"saveat", "final"}:
        raise NotImplementedError("output_when must be 'saveat' or 'final'")
    if output == "selected" and output_indices is None:
        raise ValueError("output='selected' requires output_indices")
    if output != "selected" and output_indices is not None:
        raise ValueError("output_indices is only valid with output='selected'")
    if output in WEIGHTED_OUTPUTS and integral_weights is None:
        raise ValueError(f"output={output!r} requires integral_weights")
    if output not in WEIGHTED_OUTPUTS and integral_weights is not None:
        raise ValueError("integral_weights are only valid with weighted output modes")
    if output in RATE_OUTPUTS and output_when != "saveat":
        raise ValueError(f"output={output!r} requires output_when='saveat'")
    if output in RATE_OUTPUTS and saveat is None:
        raise ValueError(f"output={output!r} requires explicit saveat values")
    if len(t_span) != 2:
        raise ValueError("t_span must contain exactly two values")
    span = (float(t_span[0]), float(t_span[1]))
    prepared.check_execution_mode(execution_mode)
    rho = np.asarray(rho0, dtype=np.complex128)
    packed = prepared.layout.pack(rho) if rho.ndim == 2 else np.asarray(rho0, dtype=np.float64)
    saveat_values = _normalize_saveat(saveat, span, save_start)
    if not dense_output and output_when == "saveat" and saveat_values is not None:
        interior = saveat_values[~np.isclose(saveat_values, span[0]) & ~np.isclose(saveat_values, span[1])]
        if interior.size:
            raise ValueError("dense_output=False cannot be used with interior saveat points")
    event_spec = normalize_stop_event(stop_event, prepared)
    eff_saveat, eff_ss = saveat_values, save_start
    if output_when == "final" and output not in INTEGRAL_OUTPUTS:
        eff_saveat = np.array([span[1]], dtype=np.float64)
        eff_ss = False
    start = time.perf_counter()
    times, values, width, solver_stats = native_api.solve_lindblad_ode_py(
        prepared.rust_plan, packed, span[0], span[1], float(abstol), float(reltol), float(dt),
        None if eff_saveat is None else np.asarray(eff_saveat, dtype=np.float64), bool(eff_ss), int(maxiters),
        execution_mode, solver, output, None if output_indices is None else list(output_indices), output_when,
        None if integral_weights is None else list(integral_weights), event_spec, bool(use_split_input_rhs),
        precision=precision,
    )
    elapsed = time.perf_counter() - start
    times = np.asarray(times, dtype=np.float64)
    stats = _stats(solver_stats, solver=solver, saved_points=times.size, elapsed=elapsed) if collect_stats else None
    if stats is not None and stats.get("event_triggered") and event_spec is not None:
        stats["event_name"] = event_spec.get("name", "event")
    if output == "full":
        return LindbladResult(t=times, packed_y=np.asarray(values, dtype=np.float64).reshape(times.size, width),
                              layout=prepared.layout, solver_stats=stats)
    if output in WEIGHTED_OUTPUTS:
        arr = np.asarray(values, dtype=np.float64)
        if output_when == "saveat" and times.size > 0:
            arr = arr.reshape(times.size, width)
        return LindbladObservableResult(t=times, values=arr, output=output, solver_stats=stats)
    arr = np.asarray(values, dtype=np.float64 if output == "populations" else np.complex128)
    if times.size > 0 and width > 0:
        arr = arr.reshape(times.size, width)
        if output_when == "final":
            arr = arr.reshape(width)
    return LindbladObservableResult(t=times, values=arr, output=output,
                                    output_indices=None if output_indices is None else list(output_indices),
                                    solver_stats=stats)


def _slot_name(slot) -> str:
    return slot.name if hasattr(slot, "name") and not isinstance(slot, str) else str(slot)


def _slot_indices(prepared: PreparedProblem, parameter_slots) -> list[int]:
    """batch.py:92-112: only base parameters are scannable."""
    if parameter_slots is None:
        return []
    names = list(prepared.parameter_graph["slot_names"])
    base_count = len(prepared.parameter_graph["base_values"])
    out = []
    for slot in parameter_slots:
        name = _slot_name(slot)
        try:
            index = names.index(name)
        except ValueError as exc:
            raise ValueError(f"unknown parameter slot {name!r}") from exc
        if index >= base_count:
            raise ValueError(f"parameter slot {name!r} is a compound parameter; only base parameters can be scanned")
        out.append(index)
    return out


def _pack_batch(prepared: PreparedProblem, rho0_batch) -> np.ndarray:
    batch = np.asarray(rho0_batch)
    if batch.ndim == 2:
        packed = np.asarray(batch, dtype=np.float64)
        if packed.shape[1] != prepared.layout.packed_len:
            raise ValueError(
                "2D rho0_batch must have shape (n_trajectories, packed_len); "
                f"expected packed_len={prepared.layout.packed_len}, got {packed.shape[1]}"
            )
        return np.ascontiguousarray(packed)
    if batch.ndim != 3:
        raise ValueError("rho0_batch must have shape (n_trajectories, packed_len) or (n_trajectories, n_states, n_states)")
    if batch.shape[1:] != (prepared.layout.n, prepared.layout.n):
        raise ValueError(f"matrix rho0_batch must have shape (n_trajectories, {prepared.layout.n}, {prepared.layout.n})")
    return np.ascontiguousarray(np.stack([prepared.layout.pack(r) for r in np.asarray(batch, dtype=np.complex128)]))


def _validate_batch_outputs(output, output_indices, integral_weights, output_when, saveat, stop_event, threads, what):
    if output not in {"populations", "selected", *WEIGHTED_OUTPUTS}:
        raise NotImplementedError(
            f"{what} currently supports output='populations', 'selected', "
            "'weighted_integral', 'photon_integral', 'excited_population', "
            "'weighted_rate', 'photon_rate', or 'excited_population_rate'"
        )
    if output == "selected" and output_indices is None:
        raise ValueError("output='selected' requires output_indices")
    if output != "selected" and output_indices is not None:
        raise ValueError("output_indices is only valid with output='selected'")
    if output in WEIGHTED_OUTPUTS and integral_weights is None:
        raise ValueError(f"output={output!r} requires integral_weights")
    if output not in WEIGHTED_OUTPUTS and integral_weights is not None:
        raise ValueError("integral_weights are only valid with weighted output modes")
    if output_when not in {"final", "saveat"}:
        raise ValueError("output_when must be 'final' or 'saveat'")
    if output_when == "saveat" and saveat is None:
        raise ValueError(f"{'batch' if what == 'batch solving' else what} output_when='saveat' requires explicit saveat values")
    if stop_event is not None and output_when != "final":
        raise ValueError(f"{'batch' if what == 'batch solving' else what} stop_event is only supported with output_when='final'")
    if output in RATE_OUTPUTS and output_when != "saveat":
        raise ValueError(f"output={output!r} requires output_when='saveat'")
    if threads is not None and threads <= 0:
        raise ValueError("threads must be positive when provided")


def solve_lindblad_batch(
    prepared: PreparedProblem,
    rho0_batch,
    t_span: Sequence[float],
    *,
    parameter_batch=None,
    parameter_slots=None,
    solver: str = "dopri5",
    execution_mode: str = "expanded_sparse",
    use_split_input_rhs: bool = True,
    abstol: float = 1e-7,
    reltol: float = 1e-4,
    dt: float = 1e-8,
    saveat=None,
    save_start: bool = True,
    maxiters: int = 100_000,
    collect_stats: bool = False,
    output: str = "populations",
    output_indices=None,
    output_when: str = "final",
    integral_weights=None,
    dense_output: bool = True,
    parallel: bool = True,
    threads: int | None = None,
    metadata: Mapping[str, Any] | None = None,
    stop_event=None,
    precision: str = "fp64",
) -> LindbladBatchResult:
    """batch.py:143-301."""
    if prepared.rust_plan is None:
        raise RuntimeError("solve_lindblad_batch requires a Rust prepared plan")
    prepared.check_execution_mode(execution_mode)
    if solver not in {"dopri5", "tsit5", "fixed_dopri5", "fixed_rk2", "fixed_rk4"}:
        raise NotImplementedError(
            "batch solving currently supports 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', and 'fixed_rk4'"
        )
    _validate_batch_outputs(output, output_indices, integral_weights, output_when, saveat, stop_event, threads, "batch solving")
    if len(t_span) != 2:
        raise ValueError("t_span must contain exactly two values")
    span = (float(t_span[0]), float(t_span[1]))
    packed = _pack_batch(prepared, rho0_batch)
    b = packed.shape[0]
    if b == 0:
        raise ValueError("rho0_batch must contain at least one trajectory")
    slot_idx = _slot_indices(prepared, parameter_slots)
    values_p = None
    if parameter_batch is not None:
        if parameter_slots is None:
            raise ValueError("parameter_slots are required when parameter_batch is provided")
        values_p = np.ascontiguousarray(parameter_batch, dtype=np.complex128)
        if values_p.shape != (b, len(slot_idx)):
            raise ValueError(f"parameter_batch must have shape ({b}, {len(slot_idx)}), got {values_p.shape}")
    elif parameter_slots is not None:
        raise ValueError("parameter_slots were provided without parameter_batch")
    saveat_values = _normalize_saveat(saveat, span, save_start)
    if not dense_output and output_when == "saveat" and saveat_values is not None:
        raise ValueError("dense_output=False is only supported with output_when='final'")
    event_spec = normalize_stop_event(stop_event, prepared)
    start = time.perf_counter()
    times, flat, width, time_count, solver_stats = native_api.solve_lindblad_batch_ode_py(
        prepared.rust_plan, packed, span[0], span[1], float(abstol), float(reltol), float(dt),
        None if saveat_values is None else np.asarray(saveat_values, dtype=np.float64), bool(save_start), int(maxiters),
        execution_mode, solver, output, None if output_indices is None else list(output_indices), output_when,
        None if integral_weights is None else list(integral_weights), slot_idx or None, values_p, bool(parallel),
        threads, event_spec, bool(use_split_input_rhs), precision=precision,
    )
    elapsed = time.perf_counter() - start
    dtype = np.float64 if output in {"populations", *WEIGHTED_OUTPUTS} else np.complex128
    vals = np.asarray(flat, dtype=dtype)
    vals = vals.reshape((b, width)) if output_when == "final" else vals.reshape((b, time_count, width))
    meta = {} if metadata is None else dict(metadata)
    if event_spec is not None:
        meta["event_triggered"] = np.asarray(solver_stats.get("event_triggered_by_trajectory", []), dtype=bool)
        meta["event_times"] = np.asarray(solver_stats.get("event_times", []), dtype=np.float64)
    return LindbladBatchResult(
        t=np.asarray(times, dtype=np.float64), values=vals, output=output,
        output_indices=None if output_indices is None else list(output_indices), trajectory_count=b,
        parameter_slots=None if parameter_slots is None else [_slot_name(s) for s in parameter_slots],
        parameter_values=values_p,
        solver_stats=_stats(solver_stats, solver=solver, saved_points=int(time_count), elapsed=elapsed) if collect_stats else None,
        metadata=meta,
    )


def initial_condition_scan(prepared: PreparedProblem, rho0_batch, t_span, **kwargs) -> LindbladBatchResult:
    """batch.py:304-310."""
    return solve_lindblad_batch(prepared, rho0_batch, t_span, **kwargs)


def parameter_scan(prepared: PreparedProblem, rho0, t_span, *, parameter_slots, parameter_batch, **kwargs) -> LindbladBatchResult:
    """batch.py:313-340: one rho0 repeated over the parameter rows."""
    values = np.asarray(parameter_batch, dtype=np.complex128)
    if values.ndim != 2:
        raise ValueError("parameter_batch must be 2D")
    rho = np.asarray(rho0)
    if rho.ndim == 1:
        packed = np.asarray(rho, dtype=np.float64)
    elif rho.ndim == 2:
        packed = prepared.layout.pack(np.asarray(rho, dtype=np.complex128))
    else:
        raise ValueError("rho0 must be a packed vector or density matrix")
    batch = np.repeat(packed.reshape(1, -1), values.shape[0], axis=0)
    return solve_lindblad_batch(prepared, batch, t_span, parameter_slots=parameter_slots, parameter_batch=values, **kwargs)


def grid_scan(prepared: PreparedProblem, rho0, t_span, *, scan: Mapping[Any, Any], **kwargs) -> LindbladBatchResult:
    """batch.py:343-519: a row-major grid, last axis fastest."""
    if not scan:
        raise ValueError("scan must contain at least one parameter")
    parameter_slots = list(scan)
    names = [_slot_name(s) for s in parameter_slots]
    axes = [np.asarray(v, dtype=np.complex128).reshape(-1) for v in scan.values()]
    if any(a.size == 0 for a in axes):
        raise ValueError("scan axes must be non-empty")
    slot_idx = _slot_indices(prepared, parameter_slots)
    rho = np.asarray(rho0)
    if rho.ndim == 1:
        packed = np.asarray(rho, dtype=np.float64)
        if packed.size != prepared.layout.packed_len:
            raise ValueError(f"packed rho0 must have length {prepared.layout.packed_len}, got {packed.size}")
    elif rho.ndim == 2:
        packed = prepared.layout.pack(np.asarray(rho, dtype=np.complex128))
    else:
        raise ValueError("rho0 must be a packed vector or density matrix")
    if len(t_span) != 2:
        raise ValueError("t_span must contain exactly two values")
    span = (float(t_span[0]), float(t_span[1]))
    save_start = bool(kwargs.pop("save_start", True))
    saveat_values = _normalize_saveat(kwargs.pop("saveat", None), span, save_start)
    solver = kwargs.pop("solver", "dopri5")
    execution_mode = kwargs.pop("execution_mode", "expanded_sparse")
    use_split = bool(kwargs.pop("use_split_input_rhs", True))
    abstol = float(kwargs.pop("abstol", 1e-7))
    reltol = float(kwargs.pop("reltol", 1e-4))
    dt = float(kwargs.pop("dt", 1e-8))
    maxiters = int(kwargs.pop("maxiters", 100_000))
    collect_stats = bool(kwargs.pop("collect_stats", False))
    output = kwargs.pop("output", "populations")
    output_indices = kwargs.pop("output_indices", None)
    output_when = kwargs.pop("output_when", "final")
    integral_weights = kwargs.pop("integral_weights", None)
    dense_output = bool(kwargs.pop("dense_output", True))
    parallel = bool(kwargs.pop("parallel", True))
    threads = kwargs.pop("threads", None)
    metadata = kwargs.pop("metadata", None)
    stop_event = kwargs.pop("stop_event", None)
    precision = kwargs.pop("precision", "fp64")
    if kwargs:
        raise TypeError(f"unexpected grid_scan keyword argument(s): {', '.join(sorted(kwargs))}")
    if prepared.rust_plan is None:
        raise RuntimeError("grid_scan requires a Rust prepared plan")
    prepared.check_execution_mode(execution_mode)
    if solver not in {"dopri5", "tsit5", "fixed_dopri5", "fixed_rk2", "fixed_rk4"}:
        raise NotImplementedError("grid_scan currently supports 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', and 'fixed_rk4'")
    _validate_batch_outputs(output, output_indices, integral_weights, output_when, saveat_values, stop_event, threads, "grid_scan")
    if not dense_output and output_when == "saveat" and saveat_values is not None:
        raise ValueError("dense_output=False is only supported with output_when='final'")
    lengths = [int(a.size) for a in axes]
    count = int(np.prod(lengths, dtype=np.int64))
    event_spec = normalize_stop_event(stop_event, prepared)
    start = time.perf_counter()
    times, flat, width, time_count, solver_stats = native_api.solve_lindblad_grid_ode_py(
        prepared.rust_plan, np.ascontiguousarray(packed, dtype=np.float64), span[0], span[1], abstol, reltol, dt,
        slot_idx, np.ascontiguousarray(np.concatenate(axes)), lengths,
        None if saveat_values is None else np.asarray(saveat_values, dtype=np.float64), save_start, maxiters,
        execution_mode, solver, output, None if output_indices is None else list(output_indices), output_when,
        None if integral_weights is None else list(integral_weights), parallel, threads, event_spec, use_split,
        precision=precision,
    )
    elapsed = time.perf_counter() - start
    dtype = np.float64 if output in {"populations", *WEIGHTED_OUTPUTS} else np.complex128
    vals = np.asarray(flat, dtype=dtype)
    vals = vals.reshape((count, width)) if output_when == "final" else vals.reshape((count, time_count, width))
    meta = {} if metadata is None else dict(metadata)
    if event_spec is not None:
        meta["event_triggered"] = np.asarray(solver_stats.get("event_triggered_by_trajectory", []), dtype=bool)
        meta["event_times"] = np.asarray(solver_stats.get("event_times", []), dtype=np.float64)
    result = LindbladBatchResult(
        t=np.asarray(times, dtype=np.float64), values=vals, output=output,
        output_indices=None if output_indices is None else list(output_indices), trajectory_count=count,
        parameter_slots=names, parameter_values=None,
        solver_stats=_stats(solver_stats, solver=solver, saved_points=int(time_count), elapsed=elapsed) if collect_stats else None,
        metadata=meta,
    )
    result.metadata.update({
        "scan_kind": "grid",
        "grid_shape": tuple(lengths),
        "grid_axes": dict(zip(names, axes, strict=True)),
        "compact_grid": True,
    })
    return result
