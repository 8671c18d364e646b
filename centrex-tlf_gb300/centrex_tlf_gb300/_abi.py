"""ctypes mirror of include/obe_gb300.h and the loader of the in-tree native library.

The structures here match the C declarations field for field; ``load_library`` opens
``_lib/libobe_gb300.so`` (built by ``centrex_tlf_gb300.build``) and fails loudly when it is
missing: there is no CPU fallback for the solver.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

PACKAGE_DIR = Path(__file__).resolve().parent
LIB_DIR = PACKAGE_DIR / "_lib"
LIB_PATH = LIB_DIR / "libobe_gb300.so"

OBE_OK = 0
OBE_ERR_INVALID = 1
OBE_ERR_TRAJECTORY = 2
OBE_ERR_UNSUPPORTED = 3
OBE_ERR_CUDA = 4
OBE_ERR_TIMEOUT = 5

SOLVERS = {"dopri5": 0, "tsit5": 1, "fixed_dopri5": 2, "fixed_rk2": 3, "fixed_rk4": 4}
OUTPUT_POPULATIONS = 0
OUTPUT_SELECTED = 1
OUTPUT_FULL = 2
OUTPUT_WEIGHTED_INTEGRAL = 3
OUTPUT_WEIGHTED_RATE = 4
EVENT_NONE = 0
EVENT_POPULATION = 1
EVENT_EXPRESSION = 2
PRECISIONS = {"fp64": 0, "mixed": 1, "mixed_fp32_control": 2}

_p = ctypes.POINTER
c_i32p = _p(ctypes.c_int32)
c_i64p = _p(ctypes.c_int64)
c_f64p = _p(ctypes.c_double)
c_u8p = _p(ctypes.c_uint8)


class ObeExpr(ctypes.Structure):
    _fields_ = [
        ("n_instr", ctypes.c_int64),
        ("op", c_i32p),
        ("index", c_i64p),
        ("argc", c_i32p),
        ("function", c_i32p),
        ("value", c_f64p),
        ("scalar_only", ctypes.c_int32),
        ("output_is_tuple", ctypes.c_int32),
    ]


class ObePlanDesc(ctypes.Structure):
    _fields_ = [
        ("n_states", ctypes.c_int32),
        ("n_slots", ctypes.c_int32),
        ("n_base", ctypes.c_int32),
        ("base_is_tuple", c_i32p),
        ("base_scalar", c_f64p),
        ("base_tuple_ptr", c_i64p),
        ("base_tuple_items", c_f64p),
        ("n_compounds", ctypes.c_int32),
        ("compound_slot", c_i32p),
        ("compound_expr", _p(ObeExpr)),
        ("n_pchip", ctypes.c_int32),
        ("pchip_ptr", c_i64p),
        ("pchip_grid", c_f64p),
        ("pchip_values", c_f64p),
        ("hamiltonian_decomposed", ctypes.c_int32),
        ("n_coefficients", ctypes.c_int32),
        ("coefficient_expr", _p(ObeExpr)),
        ("has_expanded", ctypes.c_int32),
        ("n_terms", ctypes.c_int64),
        ("output_ptrs", c_i64p),
        ("input_indices", c_i64p),
        ("coeff_indices", c_i64p),
        ("coeff_conj", c_u8p),
        ("input_conj", c_u8p),
        ("factors_re", c_f64p),
        ("factors_im", c_f64p),
        ("source_decay_rates", c_f64p),
    ]


class ObeSolveOptions(ctypes.Structure):
    _fields_ = [
        ("t0", ctypes.c_double),
        ("t1", ctypes.c_double),
        ("abstol", ctypes.c_double),
        ("reltol", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("maxiters", ctypes.c_int64),
        ("solver", ctypes.c_int32),
        ("save_start", ctypes.c_int32),
        ("has_saveat", ctypes.c_int32),
        ("n_saveat", ctypes.c_int64),
        ("saveat", c_f64p),
        ("output", ctypes.c_int32),
        ("store_trace", ctypes.c_int32),
        ("n_weights", ctypes.c_int32),
        ("weight_index", c_i64p),
        ("weight_value", c_f64p),
        ("n_selected", ctypes.c_int32),
        ("selected_i", c_i64p),
        ("selected_j", c_i64p),
        ("event_kind", ctypes.c_int32),
        ("n_event_indices", ctypes.c_int32),
        ("event_indices", c_i64p),
        ("event_threshold", ctypes.c_double),
        ("event_expr", ObeExpr),
        ("precision", ctypes.c_int32),
    ]


class ObeTrajStats(ctypes.Structure):
    _fields_ = [
        ("accepted_steps", ctypes.c_int64),
        ("rejected_steps", ctypes.c_int64),
        ("rhs_calls", ctypes.c_int64),
        ("event_triggered", ctypes.c_int32),
        ("status", ctypes.c_int32),
        ("event_time", ctypes.c_double),
        ("n_points", ctypes.c_int64),
    ]


class ObeInterpOperator(ctypes.Structure):
    """obe_interp_operator: a CSR matrix whose entries are cubics in the field coordinate."""

    _fields_ = [("row_ptrs", c_i64p), ("col_indices", c_i64p), ("coeffs", c_f64p), ("nnz", ctypes.c_int64)]


class ObeEffectiveDesc(ctypes.Structure):
    """obe_effective_desc: the operators and slots of an interpolated effective-Hamiltonian plan."""

    _fields_ = [
        ("real_dim", ctypes.c_int64),
        ("n_grid", ctypes.c_int32),
        ("field_grid", c_f64p),
        ("combined", ObeInterpOperator),
        ("optical", ObeInterpOperator),
        ("detuning", ObeInterpOperator),
        ("field_slot", ctypes.c_int32),
        ("rabi_slot", ctypes.c_int32),
        ("detuning_slot", ctypes.c_int32),
    ]


class ObeBatchJob(ctypes.Structure):
    """obe_batch_job: one device-resident batch of obe_solve_multi_device."""

    _fields_ = [
        ("plan", ctypes.c_void_p),
        ("opt", ctypes.POINTER(ObeSolveOptions)),
        ("n_traj", ctypes.c_int64),
        ("d_rho0", ctypes.c_void_p),
        ("n_param_slots", ctypes.c_int32),
        ("param_slots", c_i64p),
        ("d_param_values", ctypes.c_void_p),
        ("time_count", ctypes.c_int64),
        ("width", ctypes.c_int64),
        ("d_values", ctypes.c_void_p),
        ("d_stats", ctypes.c_void_p),
    ]


MAX_JOBS = 16  # OBE_MAX_JOBS


# numpy view of obe_traj_stats (same layout: 8+8+8+4+4+8+8 = 48 bytes, naturally aligned)
TRAJ_STATS_DTYPE = np.dtype(
    [
        ("accepted_steps", "<i8"),
        ("rejected_steps", "<i8"),
        ("rhs_calls", "<i8"),
        ("event_triggered", "<i4"),
        ("status", "<i4"),
        ("event_time", "<f8"),
        ("n_points", "<i8"),
    ]
)
assert TRAJ_STATS_DTYPE.itemsize == ctypes.sizeof(ObeTrajStats)


def ptr(arr: np.ndarray | None, ctype):
    """Pointer to a contiguous numpy array's data (NULL for None)."""
    if arr is None:
        return ctypes.cast(None, ctypes.POINTER(ctype))
    if not arr.flags["C_CONTIGUOUS"]:
        raise ValueError("internal error: array passed to the native library is not contiguous")
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


_LIB = None


class NativeLibraryMissing(RuntimeError):
    """Raised when the CUDA solver library has not been built."""


def load_library() -> ctypes.CDLL:
    """Open the in-tree CUDA solver library; raise if it is absent (no fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise NativeLibraryMissing(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(the GB300 solver has no CPU fallback)"
        )
    lib = ctypes.CDLL(str(LIB_PATH))
    lib.obe_last_error.restype = ctypes.c_char_p
    lib.obe_abi_version.restype = ctypes.c_int32
    lib.obe_device_count.restype = ctypes.c_int32
    lib.obe_plan_create.argtypes = [ctypes.POINTER(ObePlanDesc), ctypes.POINTER(ctypes.c_void_p)]
    lib.obe_plan_create.restype = ctypes.c_int
    lib.obe_plan_destroy.argtypes = [ctypes.c_void_p]
    lib.obe_plan_destroy.restype = None
    lib.obe_plan_packed_len.argtypes = [ctypes.c_void_p]
    lib.obe_plan_packed_len.restype = ctypes.c_int64
    lib.obe_plan_n_states.argtypes = [ctypes.c_void_p]
    lib.obe_plan_n_states.restype = ctypes.c_int32
    lib.obe_plan_trace_preserving.argtypes = [ctypes.c_void_p]
    lib.obe_plan_trace_preserving.restype = ctypes.c_int32
    lib.obe_dense_commutator_tf32.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.obe_dense_commutator_tf32.restype = ctypes.c_int
    lib.obe_rhs_eval.argtypes = [
        ctypes.c_void_p, ctypes.c_int64, c_f64p, c_f64p, ctypes.c_int32, c_i64p, c_f64p,
        ctypes.c_int32, c_f64p,
    ]
    lib.obe_rhs_eval.restype = ctypes.c_int
    lib.obe_solve_single.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(ObeSolveOptions), c_f64p, ctypes.POINTER(ctypes.c_void_p)
    ]
    lib.obe_solve_single.restype = ctypes.c_int
    lib.obe_result_shape.argtypes = [ctypes.c_void_p, c_i64p, c_i64p, c_i32p]
    lib.obe_result_shape.restype = None
    lib.obe_result_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ObeTrajStats)]
    lib.obe_result_stats.restype = None
    lib.obe_result_copy.argtypes = [ctypes.c_void_p, c_f64p, c_f64p]
    lib.obe_result_copy.restype = None
    lib.obe_result_destroy.argtypes = [ctypes.c_void_p]
    lib.obe_result_destroy.restype = None
    lib.obe_solve_batch.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(ObeSolveOptions), ctypes.c_int64, c_f64p, ctypes.c_int32,
        c_i64p, c_f64p, ctypes.c_int64, ctypes.c_int64, c_f64p, ctypes.c_void_p,
    ]
    lib.obe_solve_batch.restype = ctypes.c_int
    lib.obe_solve_grid.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(ObeSolveOptions), c_f64p, ctypes.c_int32, c_i64p, c_i64p,
        c_f64p, ctypes.c_int64, ctypes.c_int64, c_f64p, ctypes.c_void_p,
    ]
    lib.obe_solve_grid.restype = ctypes.c_int
    lib.obe_solve_batch_device.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(ObeSolveOptions), ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_int32, c_i64p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p,
    ]
    lib.obe_solve_batch_device.restype = ctypes.c_int
    lib.obe_last_launch_count.restype = ctypes.c_int64
    lib.obe_solve_multi_device.argtypes = [ctypes.c_int32, ctypes.POINTER(ObeBatchJob), ctypes.c_void_p]
    lib.obe_solve_multi_device.restype = ctypes.c_int
    lib.obe_multi_graph_create.argtypes = [ctypes.c_int32, ctypes.POINTER(ObeBatchJob), ctypes.POINTER(ctypes.c_void_p)]
    lib.obe_multi_graph_create.restype = ctypes.c_int
    lib.obe_multi_graph_launch.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.obe_multi_graph_launch.restype = ctypes.c_int
    lib.obe_multi_graph_destroy.argtypes = [ctypes.c_void_p]
    lib.obe_multi_graph_destroy.restype = None
    lib.obe_effective_plan_create.argtypes = [ctypes.POINTER(ObePlanDesc), ctypes.POINTER(ObeEffectiveDesc),
                                              ctypes.POINTER(ctypes.c_void_p)]
    lib.obe_effective_plan_create.restype = ctypes.c_int
    lib.obe_effective_rhs_debug.argtypes = [ctypes.c_void_p, ctypes.c_double, c_f64p, c_f64p, c_f64p]
    lib.obe_effective_rhs_debug.restype = ctypes.c_int
    lib.obe_plan_set_shape.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]
    lib.obe_plan_set_shape.restype = ctypes.c_int
    lib.obe_plan_get_shape.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    lib.obe_plan_get_shape.restype = None
    lib.obe_plan_autotune.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(ObeSolveOptions), ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, c_i64p,
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
        ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float),
        ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p,
    ]
    lib.obe_plan_autotune.restype = ctypes.c_int
    lib.obe_grad_tape_doubles_per_step.argtypes = [ctypes.c_void_p]
    lib.obe_grad_tape_doubles_per_step.restype = ctypes.c_int64
    lib.obe_grad_tape_doubles.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32]
    lib.obe_grad_tape_doubles.restype = ctypes.c_int64
    lib.obe_grad_tape_doubles_per_step_for.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.obe_grad_tape_doubles_per_step_for.restype = ctypes.c_int64
    lib.obe_grad_tape_doubles_for.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32]
    lib.obe_grad_tape_doubles_for.restype = ctypes.c_int64
    lib.obe_grad_forward.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(ObeSolveOptions), ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, c_i64p,
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p,
    ]
    lib.obe_grad_forward.restype = ctypes.c_int
    lib.obe_grad_backward.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(ObeSolveOptions), ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, c_i64p,
        ctypes.c_void_p, ctypes.c_int32, c_i64p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
    ]
    lib.obe_grad_backward.restype = ctypes.c_int
    _LIB = lib
    return lib


def last_error(lib) -> str:
    msg = lib.obe_last_error()
    return msg.decode("utf-8", "replace") if msg else ""
