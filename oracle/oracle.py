"""ctypes front end of the CPU oracle (oracle/obe_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, ``__graft_entry__.smoke()`` and the benchmark's CPU legs
use it as the parity checker and as the timed CPU baseline.  The product never imports it.

The oracle restates the reference's Rust FP64 solver (rust/src/lindblad, rust/src/ode) in C;
this module builds it on first use (``make`` in this directory) and exposes the same plan
payload / options conventions as the GPU library.
"""

from __future__ import annotations

import ctypes
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
LIB_PATH = HERE / "_build" / "libobe_oracle.so"
sys.path.insert(0, str(REPO / "centrex-tlf_gb300"))

from centrex_tlf_gb300 import _abi  # noqa: E402
from centrex_tlf_gb300._abi import ObePlanDesc, ObeSolveOptions, ObeTrajStats  # noqa: E402
from centrex_tlf_gb300._options import SolveOptions  # noqa: E402
from centrex_tlf_gb300._plan import PlanArrays  # noqa: E402

_LIB = None


def build() -> Path:
    subprocess.run(["make", "-s"], cwd=HERE, check=True)
    return LIB_PATH


def _lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        build()
    lib = ctypes.CDLL(str(LIB_PATH))
    vp = ctypes.c_void_p
    f64p, i64p = _abi.c_f64p, _abi.c_i64p
    lib.orc_plan_create.argtypes = [ctypes.POINTER(ObePlanDesc), ctypes.c_char_p, ctypes.c_size_t]
    lib.orc_plan_create.restype = vp
    lib.orc_plan_destroy.argtypes = [vp]
    lib.orc_plan_destroy.restype = None
    lib.orc_rhs.argtypes = [vp, ctypes.c_int32, i64p, f64p, ctypes.c_double, f64p, f64p, ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t]
    lib.orc_rhs.restype = ctypes.c_int
    lib.orc_coefficients.argtypes = [vp, ctypes.c_int32, i64p, f64p, ctypes.c_double, f64p, ctypes.c_char_p, ctypes.c_size_t]
    lib.orc_coefficients.restype = ctypes.c_int
    lib.orc_solve_batch.argtypes = [
        vp, ctypes.POINTER(ObeSolveOptions), ctypes.c_int64, f64p, ctypes.c_int64, ctypes.c_int32, i64p, f64p,
        ctypes.c_int64, ctypes.c_int64, f64p, f64p, vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t,
    ]
    lib.orc_solve_batch.restype = ctypes.c_int
    lib.orc_solve_single.argtypes = [
        vp, ctypes.POINTER(ObeSolveOptions), f64p, ctypes.c_int32, i64p, f64p, ctypes.c_int64, f64p, f64p,
        ctypes.POINTER(ObeTrajStats), ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t,
    ]
    lib.orc_solve_single.restype = ctypes.c_int
    lib.orc_max_threads.restype = ctypes.c_int32
    lib.orc_effective_plan_create.argtypes = [ctypes.POINTER(ObePlanDesc), ctypes.POINTER(_abi.ObeEffectiveDesc),
                                              ctypes.c_char_p, ctypes.c_size_t]
    lib.orc_effective_plan_create.restype = vp
    lib.orc_solve_replay.argtypes = [
        vp, ctypes.POINTER(ObeSolveOptions), ctypes.c_int64, f64p, ctypes.c_int64, ctypes.c_int32, i64p, f64p, i64p, f64p,
        ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), ctypes.c_int64, f64p, ctypes.c_char_p, ctypes.c_size_t,
    ]
    lib.orc_solve_replay.restype = ctypes.c_int
    _LIB = lib
    return lib


class OracleError(ValueError):
    pass


def max_threads() -> int:
    return int(_lib().orc_max_threads())


def _overrides(slots, values):
    slots = np.ascontiguousarray(np.asarray(slots if slots is not None else [], dtype=np.int64).reshape(-1))
    vals = np.asarray(values if values is not None else [], dtype=np.complex128).reshape(-1)
    packed = np.ascontiguousarray(np.stack([vals.real, vals.imag], axis=-1).reshape(-1)) if vals.size else np.zeros(0)
    return slots, packed


class OraclePlan:
    def __init__(self, payload: dict) -> None:
        self.arrays = PlanArrays(payload)
        err = ctypes.create_string_buffer(512)
        handle = _lib().orc_plan_create(ctypes.byref(self.arrays.desc), err, 512)
        if not handle:
            raise OracleError(err.value.decode())
        self.handle = handle
        self.n = self.arrays.n_states
        self.N = self.n * self.n
        self.slot_names = self.arrays.slot_names

    def __del__(self) -> None:
        if getattr(self, "handle", None) and _LIB is not None:
            _LIB.orc_plan_destroy(self.handle)
            self.handle = None

    def rhs(self, y, t, override_slots=None, override_values=None, use_split_input_rhs=True) -> np.ndarray:
        y = np.ascontiguousarray(y, dtype=np.float64)
        dy = np.zeros(self.N)
        slots, vals = _overrides(override_slots, override_values)
        err = ctypes.create_string_buffer(512)
        rc = _lib().orc_rhs(self.handle, int(slots.size), _abi.ptr(slots if slots.size else None, ctypes.c_int64),
                            _abi.ptr(vals if vals.size else None, ctypes.c_double), float(t),
                            _abi.ptr(y, ctypes.c_double), _abi.ptr(dy, ctypes.c_double), int(use_split_input_rhs), err, 512)
        if rc:
            raise OracleError(err.value.decode())
        return dy

    def coefficients(self, t, override_slots=None, override_values=None) -> np.ndarray:
        k = len(self.arrays.coefficient_exprs)
        out = np.zeros(2 * max(k, 1))
        slots, vals = _overrides(override_slots, override_values)
        err = ctypes.create_string_buffer(512)
        rc = _lib().orc_coefficients(self.handle, int(slots.size), _abi.ptr(slots if slots.size else None, ctypes.c_int64),
                                     _abi.ptr(vals if vals.size else None, ctypes.c_double), float(t),
                                     _abi.ptr(out, ctypes.c_double), err, 512)
        if rc:
            raise OracleError(err.value.decode())
        return out[: 2 * k].view(np.complex128)

    def options(self, **kw) -> SolveOptions:
        return SolveOptions(n_states=self.n, **kw)

    def solve_batch(self, opts: SolveOptions, rho0, param_slots=None, param_values=None, time_count=1,
                    threads=0, use_split_input_rhs=True):
        """rho0: (N,) shared or (B, N); param_values: (B, S) complex or None.
        Returns (values, times, stats)."""
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64)
        if param_values is not None:
            pv = np.asarray(param_values, dtype=np.complex128)
            b = pv.shape[0]
        else:
            pv = None
            b = rho0.shape[0] if rho0.ndim == 2 else 1
        stride = self.N if rho0.ndim == 2 else 0
        slots = np.ascontiguousarray(np.asarray(param_slots if param_slots is not None else [0], dtype=np.int64))
        n_slots = 0 if pv is None else pv.shape[1]
        pvals = np.ascontiguousarray(np.stack([pv.real, pv.imag], axis=-1).reshape(-1)) if pv is not None else None
        width = opts.width
        per = time_count * width * (2 if opts.is_complex else 1)
        values = np.zeros(b * per)
        times = np.zeros(max(time_count, 1))
        stats = np.zeros(b, dtype=_abi.TRAJ_STATS_DTYPE)
        err = ctypes.create_string_buffer(1024)
        rc = _lib().orc_solve_batch(
            self.handle, ctypes.byref(opts.opts), b, _abi.ptr(rho0, ctypes.c_double), stride, n_slots,
            _abi.ptr(slots, ctypes.c_int64), _abi.ptr(pvals, ctypes.c_double), time_count, width,
            _abi.ptr(values, ctypes.c_double), _abi.ptr(times, ctypes.c_double), stats.ctypes.data_as(ctypes.c_void_p),
            int(threads), int(use_split_input_rhs), err, 1024,
        )
        if rc:
            raise OracleError(err.value.decode())
        if opts.is_complex:
            values = values.view(np.complex128)
        return values.reshape(b, time_count, width), times[:time_count], stats

    def solve_replay(self, opts: SolveOptions, rho0, param_slots, param_values, steps, event_hit=None):
        """Replay frozen step sequences: steps[b] is an (n_b, 2) array of (t_n, h_n); event_hit[b]:
        its last step ended on opts' stop event (found again by bisection).  Returns the weighted
        integral (B,) or the final populations (B, n) of opts' output."""
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64)
        pv = np.asarray(param_values, dtype=np.complex128)
        b = pv.shape[0]
        stride = self.N if rho0.ndim == 2 else 0
        slots = np.ascontiguousarray(np.asarray(param_slots, dtype=np.int64))
        pvals = np.ascontiguousarray(np.stack([pv.real, pv.imag], axis=-1).reshape(-1))
        max_steps = max(1, max(len(s_) for s_ in steps))
        flat = np.zeros((b, max_steps, 2))
        counts = np.zeros(b, dtype=np.int64)
        for i, s_ in enumerate(steps):
            s_ = np.asarray(s_, dtype=np.float64).reshape(-1, 2)
            flat[i, : len(s_)] = s_
            counts[i] = len(s_)
        width = opts.width
        values = np.zeros(b * width)
        err = ctypes.create_string_buffer(1024)
        hits = None if event_hit is None else np.ascontiguousarray(np.asarray(event_hit, dtype=np.int32).reshape(b))
        rc = _lib().orc_solve_replay(
            self.handle, ctypes.byref(opts.opts), b, _abi.ptr(rho0, ctypes.c_double), stride, int(slots.size),
            _abi.ptr(slots, ctypes.c_int64), _abi.ptr(pvals, ctypes.c_double), _abi.ptr(counts, ctypes.c_int64),
            _abi.ptr(np.ascontiguousarray(flat.reshape(-1)), ctypes.c_double), max_steps,
            None if hits is None else hits.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), width,
            _abi.ptr(values, ctypes.c_double), err, 1024,
        )
        if rc:
            raise OracleError(err.value.decode())
        return values.reshape(b, width) if width > 1 else values

    def solve_single(self, opts: SolveOptions, rho0, param_slots=None, param_values=None, capacity=1024,
                     use_split_input_rhs=True):
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64)
        slots, vals = _overrides(param_slots, param_values)
        while True:
            width = opts.width
            times = np.zeros(capacity)
            values = np.zeros(capacity * width * (2 if opts.is_complex else 1))
            st = ObeTrajStats()
            err = ctypes.create_string_buffer(1024)
            rc = _lib().orc_solve_single(
                self.handle, ctypes.byref(opts.opts), _abi.ptr(rho0, ctypes.c_double), int(slots.size),
                _abi.ptr(slots if slots.size else None, ctypes.c_int64), _abi.ptr(vals if vals.size else None, ctypes.c_double),
                capacity, _abi.ptr(times, ctypes.c_double), _abi.ptr(values, ctypes.c_double), ctypes.byref(st),
                int(use_split_input_rhs), err, 1024,
            )
            if rc:
                raise OracleError(err.value.decode())
            if st.n_points <= capacity:
                break
            capacity = int(st.n_points) + 1
        n = int(st.n_points)
        if opts.is_complex:
            values = values.view(np.complex128)
        stats = {
            "accepted_steps": int(st.accepted_steps),
            "rejected_steps": int(st.rejected_steps),
            "rhs_calls": int(st.rhs_calls),
            "event_triggered": bool(st.event_triggered),
            "event_time": float(st.event_time),
        }
        return times[:n].copy(), values[: n * width].reshape(n, width).copy(), stats


class EffectiveOraclePlan(OraclePlan):
    """The oracle on an interpolated effective-Hamiltonian plan (the reference's plan_dict of
    prepare_effective_lindblad_plan_py): split-real state of 2 n^2 doubles, the effective API's
    output conventions."""

    def __init__(self, plan_dict: dict) -> None:
        from centrex_tlf_gb300._plan import EffectiveArrays

        self.eff = EffectiveArrays(plan_dict)
        self.arrays = self.eff.graph
        err = ctypes.create_string_buffer(512)
        handle = _lib().orc_effective_plan_create(ctypes.byref(self.eff.graph.desc), ctypes.byref(self.eff.desc), err, 512)
        if not handle:
            raise OracleError(err.value.decode())
        self.handle = handle
        self.n = self.eff.n_states
        self.N = self.eff.real_dim
        self.slot_names = self.eff.slot_names

    def options(self, **kw) -> SolveOptions:
        kw.setdefault("output_when", "saveat")
        kw.setdefault("stop_event", None)
        return SolveOptions(n_states=self.n, state_len=self.N, **kw)
