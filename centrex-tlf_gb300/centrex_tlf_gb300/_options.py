"""Build ``obe_solve_options`` (include/obe_gb300.h) from the reference's solve arguments.

The mapping from output names and ``output_when`` to an output spec follows
rust/src/lindblad/ode_batch.rs:103-163 and python_api.rs:422-528: integral outputs keep a
trace when ``output_when == "saveat"``; the caller passes the *effective* saveat/save_start
(python_api.rs:589-617 and 723-746 apply that mapping before the solve).
"""

from __future__ import annotations

import ctypes
from collections.abc import Sequence
from typing import Any

import numpy as np

from . import _abi
from ._abi import ObeSolveOptions
from ._plan import ExprArrays

INTEGRAL_OUTPUTS = ("weighted_integral", "photon_integral", "excited_population")
RATE_OUTPUTS = ("weighted_rate", "photon_rate", "excited_population_rate")


def packed_upper_real_index(n: int, i: int, j: int) -> int:
    """Packed index of Re rho_ij, i < j (python_api.rs:341-347; state_layout.py:27-33)."""
    off = 0
    for row in range(i):
        off += n - row - 1
    return n + 2 * (off + (j - i - 1))


class SolveOptions:
    """Owns the arrays an ``ObeSolveOptions`` points into."""

    def __init__(
        self,
        *,
        n_states: int,
        t0: float,
        t1: float,
        abstol: float,
        reltol: float,
        dt: float,
        saveat: np.ndarray | None,
        save_start: bool,
        maxiters: int,
        solver: str,
        output: str,
        output_indices: Sequence[tuple[int, int]] | None,
        output_when: str,
        integral_weights: Sequence[tuple[int, float]] | None,
        stop_event: dict[str, Any] | None,
        precision: str = "fp64",
        state_len: int | None = None,
    ) -> None:
        # the state vector's length: n^2 packed Hermitian, or 2 n^2 split-real (effective plans)
        state_len = n_states * n_states if state_len is None else int(state_len)
        if solver not in _abi.SOLVERS:
            raise ValueError(
                "solver must be 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', or 'fixed_rk4', "
                f"got {solver!r}"
            )
        if precision not in _abi.PRECISIONS:
            raise ValueError(f"precision must be 'fp64', 'mixed' or 'mixed_fp32_control', got {precision!r}")
        o = ObeSolveOptions()
        o.t0, o.t1 = float(t0), float(t1)
        o.abstol, o.reltol, o.dt = float(abstol), float(reltol), float(dt)
        maxiters = int(maxiters)
        if maxiters < 0:
            raise OverflowError("can't convert negative int to unsigned")
        o.maxiters = maxiters
        o.solver = _abi.SOLVERS[solver]
        o.save_start = int(bool(save_start))
        if saveat is None:
            self.saveat = np.zeros(1, dtype=np.float64)
            o.has_saveat, o.n_saveat = 0, 0
        else:
            self.saveat = np.ascontiguousarray(np.asarray(saveat, dtype=np.float64).reshape(-1))
            o.has_saveat, o.n_saveat = 1, int(self.saveat.size)
            if self.saveat.size == 0:
                self.saveat = np.zeros(1, dtype=np.float64)
        o.saveat = _abi.ptr(self.saveat, ctypes.c_double)

        self.is_complex = False
        self.weight_index = np.zeros(1, dtype=np.int64)
        self.weight_value = np.zeros(1, dtype=np.float64)
        self.sel_i = np.zeros(1, dtype=np.int64)
        self.sel_j = np.zeros(1, dtype=np.int64)
        o.n_weights = 0
        o.n_selected = 0
        o.store_trace = 0
        if output == "populations":
            o.output = _abi.OUTPUT_POPULATIONS
            self.width = n_states
        elif output == "selected":
            if output_indices is None:
                raise ValueError("output='selected' requires output_indices")
            pairs = [(int(i), int(j)) for i, j in output_indices]
            for i, j in pairs:
                if not (0 <= i < n_states and 0 <= j < n_states):
                    raise ValueError(f"output index {(i, j)} out of bounds for {n_states} states")
            o.output = _abi.OUTPUT_SELECTED
            self.sel_i = np.asarray([p[0] for p in pairs] or [0], dtype=np.int64)
            self.sel_j = np.asarray([p[1] for p in pairs] or [0], dtype=np.int64)
            o.n_selected = len(pairs)
            self.width = len(pairs)
            self.is_complex = True
        elif output in INTEGRAL_OUTPUTS or output in RATE_OUTPUTS:
            if integral_weights is None:
                raise ValueError(f"output='{output}' requires integral_weights")
            w = [(int(i), float(v)) for i, v in integral_weights]
            for i, _ in w:
                if not (0 <= i < state_len):
                    raise ValueError(f"integral weight index {i} out of bounds")
            self.weight_index = np.asarray([x[0] for x in w] or [0], dtype=np.int64)
            self.weight_value = np.asarray([x[1] for x in w] or [0.0], dtype=np.float64)
            o.n_weights = len(w)
            if output in INTEGRAL_OUTPUTS:
                o.output = _abi.OUTPUT_WEIGHTED_INTEGRAL
                o.store_trace = int(output_when == "saveat")
            else:
                o.output = _abi.OUTPUT_WEIGHTED_RATE
            self.width = 1
        elif output == "full":
            o.output = _abi.OUTPUT_FULL
            self.width = state_len
        else:
            raise ValueError(f"unknown output mode: {output!r}")
        o.weight_index = _abi.ptr(self.weight_index, ctypes.c_int64)
        o.weight_value = _abi.ptr(self.weight_value, ctypes.c_double)
        o.selected_i = _abi.ptr(self.sel_i, ctypes.c_int64)
        o.selected_j = _abi.ptr(self.sel_j, ctypes.c_int64)

        self.event_indices = np.zeros(1, dtype=np.int64)
        self.event_expr = None
        o.event_kind = _abi.EVENT_NONE
        o.n_event_indices = 0
        o.event_threshold = 0.0
        if stop_event is not None:
            kind = stop_event.get("kind")
            if kind is None:
                raise ValueError("stop_event missing kind")
            if kind == "population":
                if "indices" not in stop_event:
                    raise ValueError("population stop_event missing indices")
                if "threshold" not in stop_event:
                    raise ValueError("population stop_event missing threshold")
                idx = [int(i) for i in stop_event["indices"]]
                self.event_indices = np.asarray(idx or [0], dtype=np.int64)
                o.event_kind = _abi.EVENT_POPULATION
                o.n_event_indices = len(idx)
                o.event_threshold = float(stop_event["threshold"])
            elif kind == "runtime_expression":
                if "expression" not in stop_event:
                    raise ValueError("runtime stop_event missing expression")
                self.event_expr = ExprArrays(stop_event["expression"])
                self.event_expr.fill(o.event_expr)
                o.event_kind = _abi.EVENT_EXPRESSION
            else:
                raise ValueError(f"unknown stop_event kind {kind!r}")
        o.event_indices = _abi.ptr(self.event_indices, ctypes.c_int64)
        o.precision = _abi.PRECISIONS[precision]
        self.opts = o
