"""ctypes wrapper of the CUDA solver library (include/obe_gb300.h).

Every call goes to the GPU through ``_lib/libobe_gb300.so``; a missing library or a machine
without a CUDA device raises instead of falling back to a CPU path.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import ObeTrajStats, load_library
from ._options import SolveOptions
from ._plan import PlanArrays


class GpuSolverError(RuntimeError):
    """CUDA failure inside the solver library."""


def _raise(lib, status: int) -> None:
    msg = _abi.last_error(lib)
    if status in (_abi.OBE_ERR_INVALID, _abi.OBE_ERR_TRAJECTORY):
        raise ValueError(msg)
    if status == _abi.OBE_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise GpuSolverError(msg or f"solver library status {status}")


def _complex_pairs(values: np.ndarray) -> np.ndarray:
    v = np.ascontiguousarray(np.asarray(values, dtype=np.complex128))
    return v.view(np.float64).reshape(-1) if v.size else np.zeros(0)


class NativePlan:
    """An uploaded plan (``obe_plan``): the packed term tables plus the parameter program."""

    def __init__(self, payload: dict) -> None:
        self.lib = load_library()
        self.arrays = PlanArrays(payload)
        handle = ctypes.c_void_p()
        st = self.lib.obe_plan_create(ctypes.byref(self.arrays.desc), ctypes.byref(handle))
        if st != _abi.OBE_OK:
            msg = _abi.last_error(self.lib)
            if st == _abi.OBE_ERR_UNSUPPORTED:
                raise NotImplementedError(msg)
            raise ValueError(msg)
        self.handle = handle
        self.n_states = self.arrays.n_states
        self.packed_len = self.n_states * self.n_states
        self.slot_names = list(self.arrays.slot_names)
        self.n_base = self.arrays.n_base

    def __del__(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.obe_plan_destroy(h)
            self.handle = None

    @property
    def trace_preserving(self) -> bool:
        """The plan's RHS keeps the trace (the mixed form then renormalises it every step)."""
        return bool(self.lib.obe_plan_trace_preserving(self.handle))

    @classmethod
    def from_effective(cls, plan_dict: dict) -> "NativePlan":
        """An interpolated effective-Hamiltonian plan (obe_effective_plan_create) from the plan
        dict the reference's prepare_effective_lindblad_rust_plan builds; its state is split-real
        (2 n^2 doubles)."""
        from ._plan import EffectiveArrays

        self = cls.__new__(cls)
        self.lib = load_library()
        self.arrays = EffectiveArrays(plan_dict)
        handle = ctypes.c_void_p()
        st = self.lib.obe_effective_plan_create(ctypes.byref(self.arrays.graph.desc), ctypes.byref(self.arrays.desc),
                                                ctypes.byref(handle))
        if st != _abi.OBE_OK:
            msg = _abi.last_error(self.lib)
            if st == _abi.OBE_ERR_UNSUPPORTED:
                raise NotImplementedError(msg)
            raise ValueError(msg)
        self.handle = handle
        self.n_states = self.arrays.n_states
        self.packed_len = self.arrays.real_dim
        self.slot_names = list(self.arrays.slot_names)
        self.n_base = self.arrays.n_base
        return self

    def options(self, **kw) -> SolveOptions:
        return SolveOptions(n_states=self.n_states, state_len=self.packed_len, **kw)

    def effective_rhs_debug(self, y, t: float) -> tuple[np.ndarray, np.ndarray]:
        """One effective RHS at t: (dy, [field, rabi, detuning, interval])."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        dy = np.zeros(self.packed_len)
        info = np.zeros(4)
        st = self.lib.obe_effective_rhs_debug(self.handle, float(t), _abi.ptr(y, ctypes.c_double),
                                              _abi.ptr(dy, ctypes.c_double), _abi.ptr(info, ctypes.c_double))
        if st != _abi.OBE_OK:
            _raise(self.lib, st)
        return dy, info

    # -- RHS ------------------------------------------------------------------------------
    def rhs(self, y, t, override_slots=None, override_values=None, precision: str = "fp64") -> np.ndarray:
        y = np.ascontiguousarray(np.atleast_2d(np.asarray(y, dtype=np.float64)))
        count = y.shape[0]
        ts = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (count,)))
        slots = np.ascontiguousarray(np.asarray(override_slots if override_slots is not None else [], dtype=np.int64))
        if slots.size:
            ov = np.asarray(override_values, dtype=np.complex128).reshape(-1, slots.size)
            ov = np.ascontiguousarray(np.broadcast_to(ov, (count, slots.size)))
            ovp = _complex_pairs(ov)
        else:
            ovp = np.zeros(1)
        dy = np.zeros_like(y)
        st = self.lib.obe_rhs_eval(
            self.handle, count, _abi.ptr(ts, ctypes.c_double), _abi.ptr(y, ctypes.c_double), int(slots.size),
            _abi.ptr(slots if slots.size else np.zeros(1, np.int64), ctypes.c_int64), _abi.ptr(ovp, ctypes.c_double),
            _abi.PRECISIONS[precision], _abi.ptr(dy, ctypes.c_double),
        )
        if st != _abi.OBE_OK:
            _raise(self.lib, st)
        return dy

    # -- solves ---------------------------------------------------------------------------
    def solve_single(self, opts: SolveOptions, rho0):
        rho0 = np.ascontiguousarray(np.asarray(rho0, dtype=np.float64).reshape(-1))
        if rho0.size != self.packed_len:
            raise ValueError(f"expected {self.packed_len}, got {rho0.size}")
        res = ctypes.c_void_p()
        st = self.lib.obe_solve_single(self.handle, ctypes.byref(opts.opts), _abi.ptr(rho0, ctypes.c_double), ctypes.byref(res))
        if st != _abi.OBE_OK:
            _raise(self.lib, st)
        try:
            nt, w, cplx = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
            self.lib.obe_result_shape(res, ctypes.byref(nt), ctypes.byref(w), ctypes.byref(cplx))
            stats = ObeTrajStats()
            self.lib.obe_result_stats(res, ctypes.byref(stats))
            times = np.zeros(max(nt.value, 1))
            values = np.zeros(max(nt.value * w.value * (2 if cplx.value else 1), 1))
            self.lib.obe_result_copy(res, _abi.ptr(times, ctypes.c_double), _abi.ptr(values, ctypes.c_double))
        finally:
            self.lib.obe_result_destroy(res)
        n = nt.value
        times = times[:n]
        values = values[: n * w.value * (2 if cplx.value else 1)]
        if cplx.value:
            values = values.view(np.complex128)
        return times, values, int(w.value), _stats_dict(stats)

    def solve_batch(self, opts: SolveOptions, rho0_batch, param_slots=None, param_values=None, time_count: int = 1):
        rho0_batch = np.ascontiguousarray(np.asarray(rho0_batch, dtype=np.float64))
        if rho0_batch.ndim != 2 or rho0_batch.shape[1] != self.packed_len:
            raise ValueError(f"rho0 dim mismatch: {rho0_batch.shape[-1]} vs {self.packed_len}")
        b = rho0_batch.shape[0]
        slots = np.ascontiguousarray(np.asarray(param_slots if param_slots is not None else [], dtype=np.int64))
        pv = None
        if param_values is not None and slots.size:
            pv = np.asarray(param_values, dtype=np.complex128)
            if pv.shape != (b, slots.size):
                raise ValueError("parameter_batch shape mismatch")
            pv = _complex_pairs(pv)
        width = opts.width
        values = np.zeros(b * time_count * width * (2 if opts.is_complex else 1))
        stats = np.zeros(b, dtype=_abi.TRAJ_STATS_DTYPE)
        st = self.lib.obe_solve_batch(
            self.handle, ctypes.byref(opts.opts), b, _abi.ptr(rho0_batch, ctypes.c_double),
            int(slots.size) if pv is not None else 0, _abi.ptr(slots if slots.size else np.zeros(1, np.int64), ctypes.c_int64),
            _abi.ptr(pv, ctypes.c_double), time_count, width, _abi.ptr(values, ctypes.c_double),
            stats.ctypes.data_as(ctypes.c_void_p),
        )
        if st != _abi.OBE_OK:
            _raise(self.lib, st)
        if opts.is_complex:
            values = values.view(np.complex128)
        return values.reshape(b, time_count, width), stats

    def solve_grid(self, opts: SolveOptions, rho0, axis_slots, axes, time_count: int = 1):
        rho0 = np.ascontiguousarray(np.asarray(rho0, dtype=np.float64).reshape(-1))
        if rho0.size != self.packed_len:
            raise ValueError(f"packed rho0 must have length {self.packed_len}, got {rho0.size}")
        slots = np.ascontiguousarray(np.asarray(axis_slots, dtype=np.int64))
        lengths = np.ascontiguousarray(np.asarray([len(a) for a in axes], dtype=np.int64))
        flat = _complex_pairs(np.concatenate([np.asarray(a, dtype=np.complex128).reshape(-1) for a in axes]))
        b = int(np.prod(lengths))
        width = opts.width
        values = np.zeros(b * time_count * width * (2 if opts.is_complex else 1))
        stats = np.zeros(b, dtype=_abi.TRAJ_STATS_DTYPE)
        st = self.lib.obe_solve_grid(
            self.handle, ctypes.byref(opts.opts), _abi.ptr(rho0, ctypes.c_double), int(slots.size),
            _abi.ptr(slots, ctypes.c_int64), _abi.ptr(lengths, ctypes.c_int64), _abi.ptr(flat, ctypes.c_double),
            time_count, width, _abi.ptr(values, ctypes.c_double), stats.ctypes.data_as(ctypes.c_void_p),
        )
        if st != _abi.OBE_OK:
            _raise(self.lib, st)
        if opts.is_complex:
            values = values.view(np.complex128)
        return values.reshape(b, time_count, width), stats

    def solve_batch_device(self, opts: SolveOptions, n_traj: int, d_rho0: int, param_slots, d_param_values: int | None,
                           time_count: int, d_values: int, d_stats: int, stream: int = 0) -> None:
        """Device-resident batch: every data pointer is a device address (ints), asynchronous
        on ``stream``; per-trajectory statuses land in ``d_stats``."""
        slots = np.ascontiguousarray(np.asarray(param_slots if param_slots is not None else [0], dtype=np.int64))
        n_param = 0 if d_param_values is None else int(slots.size)
        st = self.lib.obe_solve_batch_device(
            self.handle, ctypes.byref(opts.opts), int(n_traj), ctypes.c_void_p(d_rho0), n_param,
            _abi.ptr(slots, ctypes.c_int64), ctypes.c_void_p(d_param_values or 0), time_count, opts.width,
            ctypes.c_void_p(d_values), ctypes.c_void_p(d_stats), ctypes.c_void_p(stream),
        )
        if st != _abi.OBE_OK:
            _raise(self.lib, st)

    # ---- launch shape (obe_plan_set_shape / obe_plan_get_shape / obe_plan_autotune) -------
    def set_shape(self, threads_per_trajectory: int = 0, trajectories_per_cta: int = 0) -> None:
        """Fix the launch shape of later solves (0, 0: the automatic choice)."""
        st = self.lib.obe_plan_set_shape(self.handle, int(threads_per_trajectory), int(trajectories_per_cta))
        if st != _abi.OBE_OK:
            _raise(self.lib, st)

    def shape(self) -> tuple[int, int]:
        """(threads per trajectory in use, fixed trajectories per CTA or 0 for automatic)."""
        t, g = ctypes.c_int32(), ctypes.c_int32()
        self.lib.obe_plan_get_shape(self.handle, ctypes.byref(t), ctypes.byref(g))
        return int(t.value), int(g.value)

    def autotune(self, opts: SolveOptions, n_traj: int, d_rho0: int, param_slots, d_param_values: int | None,
                 time_count: int, probe_steps: int = 64, stream: int = 0) -> list[dict]:
        """Time the candidate launch shapes on a probe of this device-resident batch and fix the
        fastest; returns every candidate with its probe time, the chosen one first."""
        slots = np.ascontiguousarray(np.asarray(param_slots if param_slots else [0], dtype=np.int64))
        n_param = 0 if d_param_values is None or not param_slots else int(slots.size)
        cap = 32
        ct, cg = (ctypes.c_int32 * cap)(), (ctypes.c_int32 * cap)()
        cm = (ctypes.c_float * cap)()
        nc = ctypes.c_int32()
        st = self.lib.obe_plan_autotune(
            self.handle, ctypes.byref(opts.opts), int(n_traj), ctypes.c_void_p(d_rho0), n_param,
            _abi.ptr(slots, ctypes.c_int64), ctypes.c_void_p(d_param_values or 0), int(time_count), opts.width,
            int(probe_steps), cap, ct, cg, cm, ctypes.byref(nc), ctypes.c_void_p(stream),
        )
        if st != _abi.OBE_OK:
            _raise(self.lib, st)
        cands = [{"threads_per_trajectory": int(ct[k]), "trajectories_per_cta": int(cg[k]), "probe_ms": float(cm[k])}
                 for k in range(min(nc.value, cap))]
        chosen = self.shape()
        cands.sort(key=lambda c: (c["threads_per_trajectory"], c["trajectories_per_cta"]) != chosen)
        return cands

    # ---- gradients (obe_grad_forward / obe_grad_backward) -------------------------------
    def grad_tape_doubles_per_step(self, precision: str = "fp64") -> int:
        """Doubles of one full-tape record of the form ``precision``."""
        return int(self.lib.obe_grad_tape_doubles_per_step_for(self.handle, _abi.PRECISIONS[precision]))

    def grad_tape_doubles(self, max_steps: int, checkpoint_every: int = 0, precision: str = "fp64") -> int:
        """Doubles of one trajectory's tape (full records, or checkpoints every C steps) of the
        form ``precision`` (the mixed form's full records are single precision)."""
        return int(self.lib.obe_grad_tape_doubles_for(self.handle, int(max_steps), int(checkpoint_every),
                                                      _abi.PRECISIONS[precision]))

    def grad_forward(self, opts: SolveOptions, n_traj: int, d_rho0: int, param_slots, d_param_values: int | None,
                     max_steps: int, d_tape: int, d_values: int, d_stats: int, stream: int = 0,
                     checkpoint_every: int = 0) -> None:
        """The batch solve (opts' precision) that records the gradient tape (device pointers)."""
        slots = np.ascontiguousarray(np.asarray(param_slots if param_slots else [0], dtype=np.int64))
        n_param = 0 if d_param_values is None else int(slots.size)
        st = self.lib.obe_grad_forward(
            self.handle, ctypes.byref(opts.opts), int(n_traj), ctypes.c_void_p(d_rho0), n_param,
            _abi.ptr(slots, ctypes.c_int64), ctypes.c_void_p(d_param_values or 0), int(max_steps), int(checkpoint_every),
            ctypes.c_void_p(d_tape), opts.width, ctypes.c_void_p(d_values), ctypes.c_void_p(d_stats), ctypes.c_void_p(stream),
        )
        if st != _abi.OBE_OK:
            _raise(self.lib, st)

    def grad_backward(self, opts: SolveOptions, n_traj: int, d_rho0: int, param_slots, d_param_values: int | None,
                      grad_slots, max_steps: int, d_tape: int, d_stats: int, d_out_grad: int, d_param_grad: int | None,
                      d_rho0_grad: int | None, d_adj_status: int, stream: int = 0, checkpoint_every: int = 0) -> None:
        """The reverse sweep over a tape of grad_forward (device pointers)."""
        slots = np.ascontiguousarray(np.asarray(param_slots if param_slots else [0], dtype=np.int64))
        n_param = 0 if d_param_values is None else int(slots.size)
        gslots = np.ascontiguousarray(np.asarray(grad_slots if len(grad_slots) else [0], dtype=np.int64))
        st = self.lib.obe_grad_backward(
            self.handle, ctypes.byref(opts.opts), int(n_traj), ctypes.c_void_p(d_rho0), n_param,
            _abi.ptr(slots, ctypes.c_int64), ctypes.c_void_p(d_param_values or 0), len(grad_slots),
            _abi.ptr(gslots, ctypes.c_int64), int(max_steps), int(checkpoint_every), ctypes.c_void_p(d_tape),
            ctypes.c_void_p(d_stats),
            ctypes.c_void_p(d_out_grad), ctypes.c_void_p(d_param_grad or 0), ctypes.c_void_p(d_rho0_grad or 0),
            ctypes.c_void_p(d_adj_status), ctypes.c_void_p(stream),
        )
        if st != _abi.OBE_OK:
            _raise(self.lib, st)

    def launches(self) -> int:
        return int(self.lib.obe_last_launch_count())


def _job_array(jobs):
    arr = (_abi.ObeBatchJob * len(jobs))()
    keep = []
    for k, (plan, opts, n_traj, d_rho0, slots, d_params, time_count, d_values, d_stats) in enumerate(jobs):
        sl = np.ascontiguousarray(np.asarray(slots if slots else [0], dtype=np.int64))
        keep.append(sl)
        n_param = 0 if d_params is None or not slots else int(sl.size)
        arr[k] = _abi.ObeBatchJob(plan.handle.value, ctypes.pointer(opts.opts), int(n_traj), d_rho0, n_param,
                                  _abi.ptr(sl, ctypes.c_int64), d_params or 0, int(time_count), opts.width,
                                  d_values, d_stats)
    return arr, keep


def multi_solve_device(jobs, stream: int = 0) -> int:
    """obe_solve_multi_device over device-resident batches on different plans.

    ``jobs``: sequence of ``(plan: NativePlan, opts: SolveOptions, n_traj, d_rho0, param_slots or
    None, d_param_values or None, time_count, d_values, d_stats)``, data pointers as ints.  The
    jobs' kernels run concurrently, asynchronous on ``stream``.  Returns the kernel launch count."""
    if not jobs:
        return 0
    lib = load_library()
    arr, _keep = _job_array(jobs)
    st = lib.obe_solve_multi_device(len(jobs), arr, ctypes.c_void_p(stream))
    if st != _abi.OBE_OK:
        _raise(lib, st)
    return int(lib.obe_last_launch_count())


class MultiGraph:
    """obe_multi_graph: the jobs of ``multi_solve_device`` recorded once as a CUDA graph; each
    ``launch(stream)`` replays the whole heterogeneous batch as one graph launch (refill the
    jobs' device inputs between launches, read their outputs after).  Holds its plans."""

    def __init__(self, jobs) -> None:
        lib = load_library()
        self._plans = [j[0] for j in jobs]
        arr, _keep = _job_array(jobs)
        h = ctypes.c_void_p()
        st = lib.obe_multi_graph_create(len(jobs), arr, ctypes.byref(h))
        if st != _abi.OBE_OK:
            _raise(lib, st)
        self.handle = h

    def launch(self, stream: int = 0) -> int:
        lib = load_library()
        st = lib.obe_multi_graph_launch(self.handle, ctypes.c_void_p(stream))
        if st != _abi.OBE_OK:
            _raise(lib, st)
        return int(lib.obe_last_launch_count())

    def close(self) -> None:
        if getattr(self, "handle", None) and self.handle.value:
            load_library().obe_multi_graph_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


def _stats_dict(st: ObeTrajStats) -> dict:
    return {
        "accepted_steps": int(st.accepted_steps),
        "rejected_steps": int(st.rejected_steps),
        "rhs_calls": int(st.rhs_calls),
        "event_triggered": bool(st.event_triggered),
        "event_time": float(st.event_time),
    }


def device_count() -> int:
    return int(load_library().obe_device_count())
