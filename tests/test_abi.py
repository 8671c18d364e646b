"""The C-ABI library loads, exports every entry point include/obe_gb300.h declares, and packs
plans on the host (no GPU needed for any of this)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from centrex_tlf_gb300 import _abi
from centrex_tlf_gb300 import centrex_tlf_rust as api
from centrex_tlf_gb300.native import NativePlan

HEADER = Path(__file__).resolve().parent.parent / "include" / "obe_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(obe_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _abi.load_library()
    names = declared_functions()
    assert "obe_solve_batch" in names and "obe_plan_create" in names
    for name in names:
        assert hasattr(lib, name), f"{name} is declared in include/obe_gb300.h but not exported"
    assert lib.obe_abi_version() == 2


def test_struct_layouts_match_header_sizes():
    # obe_traj_stats: 3*i64 + 2*i32 + f64 + i64
    assert ctypes.sizeof(_abi.ObeTrajStats) == 48
    assert _abi.TRAJ_STATS_DTYPE.itemsize == 48


@pytest.mark.parametrize("name", ["two_level", "two_level_td", "chain3", "chain45", "q1_16"])
def test_plans_pack_on_host(golden, name):
    payload = golden(f"plan_{name}")["payload"]
    plan = NativePlan(payload)
    n = payload["n_states"]
    assert plan.n_states == n
    assert plan.lib.obe_plan_packed_len(plan.handle) == n * n


def _payload(golden):
    import copy

    return copy.deepcopy(golden("plan_two_level")["payload"])


def test_payload_validation_messages_match_reference(golden):
    """plan.rs:1096-1150 messages."""
    p = _payload(golden)
    p["expanded_rhs_plan"]["output_ptrs"] = list(p["expanded_rhs_plan"]["output_ptrs"])[:-1]
    with pytest.raises(ValueError, match="expanded RHS output_ptrs must have length 4, got 3"):
        api.prepare_lindblad_problem_py(p)
    p = _payload(golden)
    p["expanded_rhs_plan"]["input_indices"] = [7] + list(p["expanded_rhs_plan"]["input_indices"])[1:]
    with pytest.raises(ValueError, match="expanded RHS input index 7 out of bounds for upper length 3"):
        api.prepare_lindblad_problem_py(p)
    p = _payload(golden)
    p["expanded_rhs_plan"]["n"] = 5
    with pytest.raises(ValueError, match="expanded RHS dimension 5 does not match n_states 2"):
        api.prepare_lindblad_problem_py(p)
    p = _payload(golden)
    p["expanded_rhs_plan"]["kind"] = "dense"
    with pytest.raises(ValueError, match="unknown expanded RHS plan kind: dense"):
        api.prepare_lindblad_problem_py(p)
    p = _payload(golden)
    del p["parameter_graph"]
    with pytest.raises(KeyError, match='missing key "parameter_graph"'):
        api.prepare_lindblad_problem_py(p)
    p = _payload(golden)
    p["hamiltonian_plan"]["kind"] = "magic"
    with pytest.raises(ValueError, match="unknown hamiltonian kind: magic"):
        api.prepare_lindblad_problem_py(p)
    p = _payload(golden)
    p["expanded_rhs_plan"]["coeff_indices"] = [3] * len(p["expanded_rhs_plan"]["coeff_indices"])
    with pytest.raises(ValueError, match="expanded RHS coefficient index 3 out of bounds for 2 coefficients"):
        api.prepare_lindblad_problem_py(p)


def test_argument_validation_before_any_device_work(golden):
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    rho0 = d["rho0_packed"]
    with pytest.raises(ValueError, match='unsupported execution mode "nope"'):
        api.solve_lindblad_ode_py(plan, rho0, 0.0, 1.0, 1e-8, 1e-6, 1e-3, mode="nope")
    with pytest.raises(NotImplementedError):
        api.solve_lindblad_ode_py(plan, rho0, 0.0, 1.0, 1e-8, 1e-6, 1e-3, mode="structured")
    with pytest.raises(ValueError, match=r"solver must be 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', or 'fixed_rk4', got \"rk45\""):
        api.solve_lindblad_ode_py(plan, rho0, 0.0, 1.0, 1e-8, 1e-6, 1e-3, solver="rk45")
    with pytest.raises(ValueError, match="output='selected' requires output_indices"):
        api.solve_lindblad_ode_py(plan, rho0, 0.0, 1.0, 1e-8, 1e-6, 1e-3, output="selected")
    with pytest.raises(ValueError, match="output='photon_integral' requires integral_weights"):
        api.solve_lindblad_ode_py(plan, rho0, 0.0, 1.0, 1e-8, 1e-6, 1e-3, output="photon_integral")
    with pytest.raises(ValueError, match="packed_rho0_batch must be 2D"):
        api.solve_lindblad_batch_ode_py(plan, rho0, 0.0, 1.0, 1e-8, 1e-6, 1e-3)
    with pytest.raises(ValueError, match="rho0 dim mismatch: 3 vs 4"):
        api.solve_lindblad_batch_ode_py(plan, np.zeros((2, 3)), 0.0, 1.0, 1e-8, 1e-6, 1e-3)
    with pytest.raises(ValueError, match="parameter_batch shape mismatch"):
        api.solve_lindblad_batch_ode_py(plan, np.zeros((2, 4)), 0.0, 1.0, 1e-8, 1e-6, 1e-3,
                                        parameter_slot_indices=[0], parameter_batch=np.zeros((3, 1), complex))
    with pytest.raises(ValueError, match="parameter grid axes must be non-empty"):
        api.solve_lindblad_grid_ode_py(plan, rho0, 0.0, 1.0, 1e-8, 1e-6, 1e-3, [0], np.zeros(0, complex), [0])
    with pytest.raises(ValueError, match=r"saveat value 2 is outside \[0, 1\]"):
        api.solve_lindblad_batch_ode_py(plan, np.zeros((1, 4)), 0.0, 1.0, 1e-8, 1e-6, 1e-3,
                                        saveat=np.array([0.5, 2.0]), output_when="saveat")


def test_empty_batch_returns_empty_result_without_device(golden):
    """Zero trajectories: the reference's batch loop runs no trajectory and returns width 0,
    time_count 0 and no times (ode_batch.rs:297-306); no device work is needed for that, so this
    runs without a GPU.  The argument checks still apply to an empty batch."""
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    times, values, width, tc, stats = api.solve_lindblad_batch_ode_py(plan, np.zeros((0, 4)), 0.0, 1.0, 1e-8, 1e-6, 1e-3)
    assert times.size == 0 and values.size == 0 and width == 0 and tc == 0
    assert stats["accepted_steps"] == 0 and stats["event_triggered_by_trajectory"] == []
    with pytest.raises(ValueError, match="rho0 dim mismatch: 3 vs 4"):
        api.solve_lindblad_batch_ode_py(plan, np.zeros((0, 3)), 0.0, 1.0, 1e-8, 1e-6, 1e-3)


def test_multi_batch_validation_before_device_work(golden):
    """The heterogeneous batch checks every job before it touches the device, and names the job."""
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    job = dict(plan=plan, packed_rho0_batch=np.zeros((2, 4)), t0=0.0, t1=1.0, abstol=1e-8, reltol=1e-6, dt=1e-3)
    with pytest.raises(ValueError, match=r"^job 1: rho0 dim mismatch: 3 vs 4$"):
        api.solve_lindblad_multi_batch_ode_py([job, dict(job, packed_rho0_batch=np.zeros((2, 3)))])
    with pytest.raises(TypeError, match=r"^job 0: unexpected arguments \['bogus'\]$"):
        api.solve_lindblad_multi_batch_ode_py([dict(job, bogus=1)])
    with pytest.raises(ValueError, match=r"^job 0: solver must be"):
        api.solve_lindblad_multi_batch_ode_py([dict(job, solver="rk45")])
    # the C entry point: one job per plan, at most OBE_MAX_JOBS jobs, nothing to do for none
    lib = _abi.load_library()
    native = plan.native
    opts = native.options(t0=0.0, t1=1.0, abstol=1e-8, reltol=1e-6, dt=1e-3, saveat=np.array([1.0]), save_start=False,
                          maxiters=1000, solver="dopri5", output="populations", output_indices=None,
                          output_when="final", integral_weights=None, stop_event=None)
    arr = (_abi.ObeBatchJob * 2)()
    for k in range(2):
        arr[k] = _abi.ObeBatchJob(native.handle.value, ctypes.pointer(opts.opts), 1, None, 0, None, None, 1,
                                  opts.width, None, None)
    assert lib.obe_solve_multi_device(2, arr, None) == _abi.OBE_ERR_INVALID
    assert _abi.last_error(lib) == "job 1: plan already used by job 0 (one job per plan)"
    assert lib.obe_solve_multi_device(_abi.MAX_JOBS + 1, arr, None) == _abi.OBE_ERR_INVALID
    assert lib.obe_solve_multi_device(0, None, None) == _abi.OBE_OK
    # the graph-recorded form validates the same way before touching the device
    h = ctypes.c_void_p()
    assert lib.obe_multi_graph_create(2, arr, ctypes.byref(h)) == _abi.OBE_ERR_INVALID and not h.value
    assert _abi.last_error(lib) == "job 1: plan already used by job 0 (one job per plan)"
    assert lib.obe_multi_graph_create(0, arr, ctypes.byref(h)) == _abi.OBE_ERR_INVALID and not h.value
    assert lib.obe_multi_graph_launch(None, None) == _abi.OBE_ERR_INVALID
    lib.obe_multi_graph_destroy(None)


def test_launch_shape_validation_on_host(golden):
    """obe_plan_set_shape accepts the compiled widths that hold the state and re-lays the plan's
    record streams out for them (host work only)."""
    q = NativePlan(golden("plan_q1_16")["payload"])
    assert q.shape() == (32, 0)
    for t, g in ((64, 0), (128, 2), (512, 1), (0, 0)):
        q.set_shape(t, g)
        assert q.shape() == ((t or 32), g)
    with pytest.raises(ValueError, match="threads per trajectory must be 0"):
        q.set_shape(48, 0)
    with pytest.raises(ValueError, match="trajectories per CTA must be non-negative"):
        q.set_shape(64, -1)
    big = NativePlan(golden("plan_chain45")["payload"])
    assert big.shape() == (128, 0)
    with pytest.raises(ValueError, match="a trajectory of 64 threads holds at most 1024 packed elements; this system has 2025"):
        big.set_shape(64, 0)
    big.set_shape(256, 0)
    assert big.shape() == (256, 0)


def test_no_cpu_fallback_without_gpu(golden):
    """Without a CUDA device the solver refuses instead of computing on the CPU."""
    if _abi.load_library().obe_device_count() > 0:
        pytest.skip("a GPU is present")
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    with pytest.raises(RuntimeError, match="no CUDA device"):
        api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, 0.5, 1e-10, 1e-8, 1e-3)


def test_packed_index_layout():
    """The packed state ABI (state_layout.py:35-47): diagonal first, then (Re, Im) of the upper
    triangle row by row; the shim's index function enumerates exactly those slots."""
    from centrex_tlf_gb300._options import packed_upper_real_index

    n = 5
    slots = [packed_upper_real_index(n, i, j) for i in range(n) for j in range(i + 1, n)]
    assert slots == list(range(n, n * n, 2))
    assert packed_upper_real_index(3, 0, 1) == 3 and packed_upper_real_index(3, 0, 2) == 5
    assert packed_upper_real_index(3, 1, 2) == 7


def test_trace_preservation_found_on_host(golden):
    """The packer finds which plans keep the trace (the mixed form renormalises those): every
    reference-built system here does; dropping the transfer of one decay channel breaks it."""
    import copy

    from centrex_tlf_gb300.native import NativePlan

    for name in ("two_level", "two_level_td", "chain3", "q1_16", "r0_39", "rc_76"):
        assert NativePlan(golden(f"plan_{name}")["payload"]).trace_preserving, name
    payload = copy.deepcopy(golden("plan_two_level")["payload"])
    e = payload["expanded_rhs_plan"]
    n = payload["n_states"]
    # the +rate rho_11 transfer into rho_00: the term of output (0, 0) whose input is (1, 1)
    diag1 = n  # upper index of (1, 1)
    terms = [t for t in range(int(e["output_ptrs"][0]), int(e["output_ptrs"][1]))
             if int(e["input_indices"][t]) == diag1 and int(e["coeff_indices"][t]) < 0]
    assert terms
    fr = np.array(e["factors_re"], dtype=float)
    fr[terms[0]] *= 0.5
    e["factors_re"] = fr
    assert not NativePlan(payload).trace_preserving
