"""Marshal a plan payload dict into the flat ``obe_plan_desc`` of include/obe_gb300.h.

The payload is the dict ``PreparedLindbladProblem.to_payload()`` returns
(centrex_tlf/lindblad/plan_static.py:58-68).  Key handling follows the reference parser
(rust/src/lindblad/plan.rs:726-860, 1069-1308): missing required keys raise ``KeyError`` with
the same ``missing key "..."`` text, unknown kinds raise ``ValueError``; the array checks
(lengths, bounds, monotonic pointers) are repeated by the native packer, which owns them.
"""

from __future__ import annotations

import ctypes
from typing import Any

import numpy as np

from . import _abi
from ._abi import ObeExpr, ObePlanDesc


def _required(d: dict, key: str) -> Any:
    if key not in d:
        raise KeyError(f'missing key "{key}"')
    return d[key]


OP_MIN, OP_MAX = 1, 19


class ExprArrays:
    """One compiled expression (centrex_tlf/lindblad/ir.py:28-47) as parallel arrays."""

    def __init__(self, payload: dict) -> None:
        instructions = list(_required(payload, "instructions"))
        n = len(instructions)
        self.op = np.zeros(max(n, 1), dtype=np.int32)
        self.index = np.zeros(max(n, 1), dtype=np.int64)
        self.argc = np.zeros(max(n, 1), dtype=np.int32)
        self.function = np.zeros(max(n, 1), dtype=np.int32)
        self.value = np.zeros(2 * max(n, 1), dtype=np.float64)
        for k, instr in enumerate(instructions):
            op = int(_required(instr, "op"))
            if op < OP_MIN or op > OP_MAX:
                raise ValueError(f"unknown instruction op {op}")
            self.op[k] = op
            self.index[k] = int(instr.get("index", 0))
            self.argc[k] = int(instr.get("argc", 0))
            self.function[k] = int(instr.get("function", 0))
            self.value[2 * k] = float(instr.get("re", 0.0))
            self.value[2 * k + 1] = float(instr.get("im", 0.0))
        self.n = n
        self.scalar_only = bool(payload.get("scalar_only", False))
        self.output_is_tuple = bool(payload.get("output_is_tuple", False))

    def fill(self, target: ObeExpr) -> None:
        target.n_instr = self.n
        target.op = _abi.ptr(self.op, ctypes.c_int32)
        target.index = _abi.ptr(self.index, ctypes.c_int64)
        target.argc = _abi.ptr(self.argc, ctypes.c_int32)
        target.function = _abi.ptr(self.function, ctypes.c_int32)
        target.value = _abi.ptr(self.value, ctypes.c_double)
        target.scalar_only = int(self.scalar_only)
        target.output_is_tuple = int(self.output_is_tuple)

    def uses_time(self) -> bool:
        return bool(np.any(self.op[: self.n] == 4))


class PlanArrays:
    """Owns every array an ``obe_plan_desc`` points into, and the descriptor itself."""

    def __init__(self, payload: dict) -> None:
        self.n_states = int(_required(payload, "n_states"))
        if self.n_states <= 0:
            raise ValueError("layout dimension must be positive")
        graph = _required(payload, "parameter_graph")
        self.slot_names = [str(s) for s in _required(graph, "slot_names")]
        base_values = list(_required(graph, "base_values"))
        self.n_base = len(base_values)
        self.base_is_tuple = np.zeros(max(self.n_base, 1), dtype=np.int32)
        self.base_scalar = np.zeros(2 * max(self.n_base, 1), dtype=np.float64)
        tuple_ptr = [0]
        tuple_items: list[float] = []
        for i, value in enumerate(base_values):
            kind = str(_required(value, "kind"))
            if kind == "scalar":
                self.base_scalar[2 * i] = float(_required(value, "re"))
                self.base_scalar[2 * i + 1] = float(_required(value, "im"))
            elif kind == "tuple":
                self.base_is_tuple[i] = 1
                for item in _required(value, "items"):
                    if str(_required(item, "kind")) != "scalar":
                        raise TypeError("nested tuple runtime values are not supported")
                    tuple_items.extend([float(_required(item, "re")), float(_required(item, "im"))])
            else:
                raise ValueError(f"unknown runtime value kind {kind}")
            tuple_ptr.append(len(tuple_items) // 2)
        self.base_tuple_ptr = np.asarray(tuple_ptr, dtype=np.int64)
        self.base_tuple_items = np.asarray(tuple_items if tuple_items else [0.0, 0.0], dtype=np.float64)

        compounds = list(_required(graph, "compounds"))
        self.compound_slot = np.asarray([int(_required(c, "slot")) for c in compounds] or [0], dtype=np.int32)
        self.compound_exprs = [ExprArrays(_required(c, "expression")) for c in compounds]
        self.compound_expr_array = (ObeExpr * max(len(compounds), 1))()
        for i, e in enumerate(self.compound_exprs):
            e.fill(self.compound_expr_array[i])

        tables = list(graph.get("pchip_tables", []) or [])
        ptr = [0]
        grid: list[float] = []
        vals: list[float] = []
        for table in tables:
            g = np.asarray(_required(table, "grid"), dtype=np.float64).reshape(-1)
            v = np.asarray(_required(table, "values"), dtype=np.float64).reshape(-1)
            if g.size != v.size:
                raise ValueError("pchip grid and values must have the same length")
            grid.extend(g.tolist())
            vals.extend(v.tolist())
            ptr.append(len(grid))
        self.pchip_ptr = np.asarray(ptr, dtype=np.int64)
        self.pchip_grid = np.asarray(grid or [0.0], dtype=np.float64)
        self.pchip_values = np.asarray(vals or [0.0], dtype=np.float64)
        self.n_pchip = len(tables)

        ham = _required(payload, "hamiltonian_plan")
        _required(ham, "n")
        kind = str(ham.get("kind", "entrywise"))
        if kind not in ("decomposed", "entrywise"):
            raise ValueError(f"unknown hamiltonian kind: {kind}")
        self.decomposed = kind == "decomposed"
        coeffs = list(_required(ham, "coefficients")) if self.decomposed else []
        self.coefficient_exprs = [ExprArrays(_required(c, "expression")) for c in coeffs]
        self.coefficient_expr_array = (ObeExpr * max(len(coeffs), 1))()
        for i, e in enumerate(self.coefficient_exprs):
            e.fill(self.coefficient_expr_array[i])

        self.source_decay_rates = np.ascontiguousarray(
            np.asarray(_required(payload, "source_decay_rates"), dtype=np.float64).reshape(-1)
        )
        if self.source_decay_rates.size != self.n_states:
            raise ValueError(
                f"source_decay_rates must have length {self.n_states}, got {self.source_decay_rates.size}"
            )
        dense = np.asarray(_required(payload, "dense_c_array"))
        if dense.ndim != 3 or dense.shape[1] != self.n_states or dense.shape[2] != self.n_states:
            raise ValueError(f"dense_c_array must have shape (n_collapse, {self.n_states}, {self.n_states})")
        _required(payload, "incoming_transfers_by_target")

        rhs = payload.get("expanded_rhs_plan")
        self.has_expanded = rhs is not None
        if self.has_expanded:
            kind = str(_required(rhs, "kind"))
            if kind != "expanded_sparse":
                raise ValueError(f"unknown expanded RHS plan kind: {kind}")
            n = int(_required(rhs, "n"))
            if n != self.n_states:
                raise ValueError(f"expanded RHS dimension {n} does not match n_states {self.n_states}")
            upper_len = n * (n + 1) // 2
            self.output_ptrs = np.asarray(_required(rhs, "output_ptrs"), dtype=np.int64).reshape(-1)
            self.input_indices = np.asarray(_required(rhs, "input_indices"), dtype=np.int64).reshape(-1)
            self.coeff_indices = np.asarray(_required(rhs, "coeff_indices"), dtype=np.int64).reshape(-1)
            self.coeff_conj = np.asarray(_required(rhs, "coeff_conj"), dtype=bool).astype(np.uint8).reshape(-1)
            self.input_conj = np.asarray(_required(rhs, "input_conj"), dtype=bool).astype(np.uint8).reshape(-1)
            self.factors_re = np.asarray(_required(rhs, "factors_re"), dtype=np.float64).reshape(-1)
            self.factors_im = np.asarray(_required(rhs, "factors_im"), dtype=np.float64).reshape(-1)
            t = self.input_indices.size
            if self.output_ptrs.size != upper_len + 1:
                raise ValueError(
                    f"expanded RHS output_ptrs must have length {upper_len + 1}, got {self.output_ptrs.size}"
                )
            if self.output_ptrs[0] != 0 or self.output_ptrs[-1] != t:
                raise ValueError("expanded RHS output_ptrs must start at 0 and end at term count")
            if np.any(np.diff(self.output_ptrs) < 0):
                raise ValueError("expanded RHS output_ptrs must be monotonic")
            if not (
                self.coeff_indices.size == t
                and self.coeff_conj.size == t
                and self.input_conj.size == t
                and self.factors_re.size == t
                and self.factors_im.size == t
            ):
                raise ValueError("expanded RHS term arrays must have matching lengths")
            self.n_terms = t
        else:
            self.n_terms = 0
            self.output_ptrs = np.zeros(1, dtype=np.int64)
            self.input_indices = self.coeff_indices = np.zeros(1, dtype=np.int64)
            self.coeff_conj = self.input_conj = np.zeros(1, dtype=np.uint8)
            self.factors_re = self.factors_im = np.zeros(1, dtype=np.float64)
        for name in ("output_ptrs", "input_indices", "coeff_indices", "coeff_conj", "input_conj", "factors_re", "factors_im"):
            arr = getattr(self, name)
            if arr.size == 0:
                arr = np.zeros(1, dtype=arr.dtype)
            setattr(self, name, np.ascontiguousarray(arr))

        d = ObePlanDesc()
        d.n_states = self.n_states
        d.n_slots = len(self.slot_names)
        d.n_base = self.n_base
        d.base_is_tuple = _abi.ptr(self.base_is_tuple, ctypes.c_int32)
        d.base_scalar = _abi.ptr(self.base_scalar, ctypes.c_double)
        d.base_tuple_ptr = _abi.ptr(self.base_tuple_ptr, ctypes.c_int64)
        d.base_tuple_items = _abi.ptr(self.base_tuple_items, ctypes.c_double)
        d.n_compounds = len(self.compound_exprs)
        d.compound_slot = _abi.ptr(self.compound_slot, ctypes.c_int32)
        d.compound_expr = ctypes.cast(self.compound_expr_array, ctypes.POINTER(ObeExpr))
        d.n_pchip = self.n_pchip
        d.pchip_ptr = _abi.ptr(self.pchip_ptr, ctypes.c_int64)
        d.pchip_grid = _abi.ptr(self.pchip_grid, ctypes.c_double)
        d.pchip_values = _abi.ptr(self.pchip_values, ctypes.c_double)
        d.hamiltonian_decomposed = int(self.decomposed)
        d.n_coefficients = len(self.coefficient_exprs)
        d.coefficient_expr = ctypes.cast(self.coefficient_expr_array, ctypes.POINTER(ObeExpr))
        d.has_expanded = int(self.has_expanded)
        d.n_terms = self.n_terms
        d.output_ptrs = _abi.ptr(self.output_ptrs, ctypes.c_int64)
        d.input_indices = _abi.ptr(self.input_indices, ctypes.c_int64)
        d.coeff_indices = _abi.ptr(self.coeff_indices, ctypes.c_int64)
        d.coeff_conj = _abi.ptr(self.coeff_conj, ctypes.c_uint8)
        d.input_conj = _abi.ptr(self.input_conj, ctypes.c_uint8)
        d.factors_re = _abi.ptr(self.factors_re, ctypes.c_double)
        d.factors_im = _abi.ptr(self.factors_im, ctypes.c_double)
        d.source_decay_rates = _abi.ptr(self.source_decay_rates, ctypes.c_double)
        self.desc = d

    @property
    def packed_len(self) -> int:
        return self.n_states * self.n_states


def _required_key(d: dict, key: str):
    if key not in d:
        raise ValueError(f"missing key: {key}")
    return d[key]


class EffectiveArrays:
    """Owns every array of an interpolated effective-Hamiltonian plan and its two descriptors:
    the parameter graph as an ``obe_plan_desc`` (no Hamiltonian coefficients, no expanded plan)
    and the operators as an ``obe_effective_desc``.  ``plan_dict`` is what the reference's
    prepare_effective_lindblad_rust_plan hands to its native prepare_effective_lindblad_plan_py
    (centrex_tlf/effective_hamiltonian/rust_plan.py:185-200; parsed in
    rust/src/effective_lindblad/plan.rs:116-203, whose error texts these checks keep)."""

    def __init__(self, plan_dict: dict) -> None:
        if "parameter_graph" not in plan_dict:
            raise ValueError("missing 'parameter_graph'")
        self.n_states = int(_required_key(plan_dict, "n_states"))
        self.real_dim = int(_required_key(plan_dict, "real_dim"))
        self.n_grid = int(_required_key(plan_dict, "n_grid"))
        self.field_grid = np.ascontiguousarray(np.asarray(_required_key(plan_dict, "field_grid"), dtype=np.float64).reshape(-1))
        for key in ("excited_indices", "ground_indices", "sink_indices"):
            _required_key(plan_dict, key)
        self.field_slot = int(_required_key(plan_dict, "field_coordinate_slot"))
        self.rabi_slot = int(_required_key(plan_dict, "rabi_rate_slot"))
        self.detuning_slot = int(_required_key(plan_dict, "detuning_slot"))
        bool(_required_key(plan_dict, "is_time_dependent"))
        if self.field_grid.size != self.n_grid:
            raise ValueError("field_grid length mismatch")
        n = self.n_states
        graph_payload = {
            "n_states": n, "parameter_graph": plan_dict["parameter_graph"],
            "hamiltonian_plan": {"kind": "decomposed", "n": n, "coefficients": []},
            "source_decay_rates": np.zeros(n), "incoming_transfers_by_target": [],
            "dense_c_array": np.zeros((0, n, n), dtype=np.complex128), "expanded_rhs_plan": None,
        }
        self.graph = PlanArrays(graph_payload)
        n_slots = len(self.graph.slot_names)
        for name, slot in (("field_coordinate", self.field_slot), ("rabi_rate", self.rabi_slot),
                           ("detuning", self.detuning_slot)):
            if not 0 <= slot < n_slots:
                raise ValueError(f"{name} slot {slot} out of range")
        self.ops = {}
        desc = _abi.ObeEffectiveDesc()
        desc.real_dim = self.real_dim
        desc.n_grid = self.n_grid
        desc.field_grid = _abi.ptr(self.field_grid, ctypes.c_double)
        for key, field in (("sparse_combined", "combined"), ("sparse_opt", "optical"), ("sparse_det", "detuning")):
            if key not in plan_dict:
                raise ValueError(f"missing sparse operator: {key}")
            op = plan_dict[key]
            rows = np.ascontiguousarray(np.asarray(_required_key(op, "row_ptrs"), dtype=np.int64).reshape(-1))
            cols = np.ascontiguousarray(np.asarray(_required_key(op, "col_indices"), dtype=np.int64).reshape(-1))
            coef = np.ascontiguousarray(np.asarray(_required_key(op, "pchip_coeffs"), dtype=np.float64).reshape(-1))
            _required_key(op, "grid")
            nnz = int(_required_key(op, "nnz"))
            if rows.size != self.real_dim + 1 or rows[0] != 0 or rows[-1] != nnz or np.any(np.diff(rows) < 0):
                raise ValueError(f"{key}: row_ptrs must be {self.real_dim + 1} monotonic offsets from 0 to nnz")
            if cols.size != nnz or (nnz and (cols.min() < 0 or cols.max() >= self.real_dim)):
                raise ValueError(f"{key}: col_indices must hold nnz indices below real_dim")
            if coef.size != max(self.n_grid - 1, 0) * nnz * 4:
                raise ValueError(f"{key}: pchip_coeffs must hold (n_grid - 1) * nnz * 4 values")
            keep = (rows, cols if cols.size else np.zeros(1, np.int64), coef if coef.size else np.zeros(1))
            self.ops[key] = keep
            target = getattr(desc, field)
            target.row_ptrs = _abi.ptr(keep[0], ctypes.c_int64)
            target.col_indices = _abi.ptr(keep[1], ctypes.c_int64)
            target.coeffs = _abi.ptr(keep[2], ctypes.c_double)
            target.nnz = nnz
        desc.field_slot = self.field_slot
        desc.rabi_slot = self.rabi_slot
        desc.detuning_slot = self.detuning_slot
        self.desc = desc
        self.slot_names = self.graph.slot_names
        self.n_base = self.graph.n_base
