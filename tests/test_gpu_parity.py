"""GPU parity: the CUDA solver (through the C ABI) against the CPU oracle and the reference's own
known answers, on the golden plans.

Tolerances: FP64 RHS vs the reference's Python RHS 1e-10 relative (different summation order
and fused multiply-adds only); whole FP64 solves vs the FP64 oracle 1e-9 absolute on
populations, since both controllers see the same error estimates up to rounding; the mixed
form (FP32 RHS products, FP64 accumulation) within 1e-6 on populations, the headline bar.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api
from centrex_tlf_gb300.native import NativePlan

pytestmark = pytest.mark.gpu

PLANS = ["two_level", "two_level_td", "chain3", "chain45", "q1_16"]


@pytest.fixture(scope="module")
def q1(golden):
    d = golden("plan_q1_16")
    return d, api.prepare_lindblad_problem_py(d["payload"]), oracle.OraclePlan(d["payload"])


def _scan_params(d, count, seed):
    gamma = d["gamma"]
    rng = np.random.default_rng(seed)
    return np.stack(
        [gamma * 10 ** rng.uniform(-1, 1, count), rng.uniform(-5, 5, count) * gamma, rng.uniform(0, np.pi, count)], axis=1
    ).astype(np.complex128)


def _slots(d, names=("rabi", "detuning", "theta")):
    return [d["payload"]["parameter_graph"]["slot_names"].index(s) for s in names]


@pytest.mark.parametrize("name", PLANS)
def test_rhs_fp64_matches_python_reference(golden, name):
    plan = NativePlan(golden(f"plan_{name}")["payload"])
    for case in golden(f"rhs_{name}")["cases"]:
        dy = plan.rhs(case["packed"], case["t"], case["override_slots"], case["override_values"])[0]
        ref = case["structured"]
        scale = float(np.max(np.abs(ref)))
        np.testing.assert_allclose(dy, ref, rtol=1e-10, atol=1e-13 * scale)


@pytest.mark.parametrize("name", PLANS)
def test_rhs_mixed_within_single_precision(golden, name):
    plan = NativePlan(golden(f"plan_{name}")["payload"])
    for case in golden(f"rhs_{name}")["cases"]:
        dy = plan.rhs(case["packed"], case["t"], case["override_slots"], case["override_values"], precision="mixed")[0]
        ref = case["structured"]
        scale = float(np.max(np.abs(ref)))
        assert np.max(np.abs(dy - ref)) <= 2e-5 * scale


def test_two_level_known_answer(golden):
    d = golden("plan_two_level")
    kat = d["kat"]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    _, v, width, st = api.solve_lindblad_ode_py(
        plan, d["rho0_packed"], 0.0, 0.5, kat["abstol"], kat["reltol"], kat["dt"], None, True, 100000,
        "expanded_sparse", "dopri5", "photon_integral", None, "final", [(1, 0.3)], None,
    )
    assert width == 1
    assert st["accepted_steps"] == 10 and st["rejected_steps"] == 0 and st["rhs_calls"] == 61
    # the reference's own kernels give 0.001068126891997914 (validation.csv:5, the value the
    # GPU reproduces to ~2e-15) and 0.0010681268919861524 (validation.csv:7, the oracle's,
    # bit for bit): summation order alone moves this integral by 1.1e-11 relative
    for ref in (kat["photon_integral"], 0.0010681268919861524):
        assert abs(v[0] - ref) <= 2e-11 * ref


def test_two_level_grid_known_answer(golden):
    d = golden("plan_two_level")
    kat = d["kat"]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    det = d["kat_grid"]["detuning"].astype(np.complex128)
    slot = d["payload"]["parameter_graph"]["slot_names"].index("delta")
    times, vals, width, tc, st = api.solve_lindblad_grid_ode_py(
        plan, d["rho0_packed"], 0.0, 0.5, kat["abstol"], kat["reltol"], kat["dt"], [slot], det, [det.size],
        output="photon_integral", integral_weights=[(1, 0.3)],
    )
    assert (st["accepted_steps"], st["rejected_steps"], st["rhs_calls"]) == (252, 0, 1537)
    assert tc == 1 and width == 1 and list(times) == [0.5]
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=0.0, t1=0.5, abstol=kat["abstol"], reltol=kat["reltol"], dt=kat["dt"], saveat=None, save_start=True,
                   maxiters=100000, solver="dopri5", output="photon_integral", output_indices=None, output_when="final",
                   integral_weights=[(1, 0.3)], stop_event=None)
    ref, _, _ = op.solve_batch(o, d["rho0_packed"], [slot], det.reshape(-1, 1))
    # ~10 coarse steps: the integral follows the step sizes, whose controller input (the
    # error estimate) cancels ~8 digits, so rounding-level differences show up at ~1e-9
    np.testing.assert_allclose(vals, ref.reshape(-1), rtol=2e-9)


@pytest.mark.parametrize("solver", ["dopri5", "tsit5"])
def test_q1_full_trajectory_matches_oracle(q1, solver):
    d, plan, op = q1
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    saveat = np.linspace(t0, t1, 41)
    times, vals, width, st = api.solve_lindblad_ode_py(plan, d["rho0_packed"], t0, t1, 1e-11, 1e-8, 1e-3 / gamma,
                                                       saveat, True, 100000, "expanded_sparse", solver, "full")
    o = op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=saveat, save_start=True,
                   maxiters=100000, solver=solver, output="full", output_indices=None, output_when="saveat",
                   integral_weights=None, stop_event=None)
    rt, rv, rst = op.solve_single(o, d["rho0_packed"])
    np.testing.assert_array_equal(times, rt)
    np.testing.assert_allclose(vals.reshape(rv.shape), rv, atol=1e-9)
    assert abs(st["accepted_steps"] - rst["accepted_steps"]) <= 0.02 * rst["accepted_steps"] + 2


def test_q1_every_step_output_and_selected(q1):
    d, plan, op = q1
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    common = dict(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma)
    # populations at every accepted step (saveat None): the point count is the step count + 1
    times, vals, width, st = api.solve_lindblad_ode_py(plan, d["rho0_packed"], t0, t1, 1e-11, 1e-8, 1e-3 / gamma,
                                                       None, True, 100000, "expanded_sparse", "dopri5", "populations")
    assert width == 16 and times.size == st["accepted_steps"] + 1
    np.testing.assert_allclose(vals.reshape(-1, 16).sum(axis=1), 1.0, atol=1e-9)
    pairs = [(0, 13), (14, 2), (5, 5)]
    saveat = np.linspace(t0, t1, 9)
    _, sel, w, _ = api.solve_lindblad_ode_py(plan, d["rho0_packed"], t0, t1, 1e-11, 1e-8, 1e-3 / gamma, saveat, True,
                                             100000, "expanded_sparse", "dopri5", "selected", pairs)
    o = op.options(saveat=saveat, save_start=True, maxiters=100000, solver="dopri5", output="selected",
                   output_indices=pairs, output_when="saveat", integral_weights=None, stop_event=None, **common)
    _, rsel, _ = op.solve_single(o, d["rho0_packed"])
    np.testing.assert_allclose(sel.reshape(rsel.shape), rsel, atol=1e-9)


def test_q1_integral_trace_final_and_rate(q1):
    d, plan, op = q1
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    w = [(13, 1.0), (14, 1.0), (15, 1.0)]
    common = dict(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma)
    for output_when, saveat in (("final", None), ("saveat", np.linspace(t0, t1, 11))):
        t, v, _, _ = api.solve_lindblad_ode_py(plan, d["rho0_packed"], t0, t1, 1e-11, 1e-8, 1e-3 / gamma, saveat, True,
                                               100000, "expanded_sparse", "tsit5", "excited_population", None,
                                               output_when, w)
        o = op.options(saveat=saveat, save_start=True, maxiters=100000, solver="tsit5", output="excited_population",
                       output_indices=None, output_when=output_when, integral_weights=w, stop_event=None, **common)
        rt, rv, _ = op.solve_single(o, d["rho0_packed"])
        np.testing.assert_allclose(t, rt, rtol=0, atol=1e-18)
        np.testing.assert_allclose(v, rv.reshape(-1), rtol=1e-8, atol=1e-16)
    saveat = np.linspace(t0, t1, 21)
    t, v, _, _ = api.solve_lindblad_ode_py(plan, d["rho0_packed"], t0, t1, 1e-11, 1e-8, 1e-3 / gamma, saveat, True,
                                           100000, "expanded_sparse", "dopri5", "excited_population_rate", None,
                                           "saveat", w)
    o = op.options(saveat=saveat, save_start=True, maxiters=100000, solver="dopri5", output="excited_population_rate",
                   output_indices=None, output_when="saveat", integral_weights=w, stop_event=None, **common)
    _, rv, _ = op.solve_single(o, d["rho0_packed"])
    np.testing.assert_allclose(v, rv.reshape(-1), atol=1e-10)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-6), ("mixed_fp32_control", 1e-6)])
def test_q1_parameter_scan_matches_oracle(q1, precision, tol):
    """The benchmark scan (Tsit5, excited-population integral and final populations) on 96
    seeded points of its distribution; both mixed forms hold the 1e-6 population bar."""
    d, plan, op = q1
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    params = _scan_params(d, 96, seed=3)
    slots = _slots(d)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), params.shape[0], axis=0)
    common = dict(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma)
    _, pops, width, tc, st = api.solve_lindblad_batch_ode_py(
        plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / gamma, solver="tsit5", output="populations",
        parameter_slot_indices=slots, parameter_batch=params, precision=precision)
    # the reference maps final populations to saveat=[t1], save_start=False (python_api.rs:589-617)
    o = op.options(saveat=np.array([t1]), save_start=False, maxiters=100000, solver="tsit5", output="populations",
                   output_indices=None, output_when="final", integral_weights=None, stop_event=None, **common)
    ref, _, rst = op.solve_batch(o, rho0, slots, params)
    pops = np.asarray(pops).reshape(params.shape[0], 16)
    err = np.max(np.abs(pops - ref.reshape(params.shape[0], 16)))
    assert err <= tol, f"max population error {err:.3e} > {tol}"
    assert abs(st["accepted_steps"] - int(rst["accepted_steps"].sum())) <= 0.05 * int(rst["accepted_steps"].sum())


def test_chain45_uses_group_of_warps(golden):
    """45 states runs with 128 threads per trajectory (the n > 40 side of the reference's
    partition gate); final populations across a detuning grid match the oracle."""
    d = golden("plan_chain45")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    slot = d["payload"]["parameter_graph"]["slot_names"].index("delta")
    det = np.array([0.0, 0.2, -0.3], dtype=np.complex128)
    _, vals, width, tc, st = api.solve_lindblad_grid_ode_py(plan, d["rho0_packed"], 0.0, 2.0, 1e-10, 1e-8, 1e-3, [slot],
                                                            det, [3], solver="dopri5", output="populations")
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=0.0, t1=2.0, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=np.array([2.0]), save_start=False,
                   maxiters=100000, solver="dopri5", output="populations", output_indices=None, output_when="final",
                   integral_weights=None, stop_event=None)
    ref, _, _ = op.solve_batch(o, d["rho0_packed"], [slot], det.reshape(-1, 1))
    np.testing.assert_allclose(np.asarray(vals).reshape(3, 45), ref.reshape(3, 45), atol=1e-9)


def test_population_stop_event(golden):
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    ev = {"kind": "population", "indices": [1], "threshold": 0.05}
    t, v, w, st = api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, 5.0, 1e-10, 1e-8, 1e-3, np.array([5.0]), False,
                                            100000, "expanded_sparse", "dopri5", "populations", None, "final", None, ev)
    assert st["event_triggered"] and st["event_index"] == 0
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=0.0, t1=5.0, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=np.array([5.0]), save_start=False,
                   maxiters=100000, solver="dopri5", output="populations", output_indices=None, output_when="final",
                   integral_weights=None, stop_event=ev)
    rt, rv, rst = op.solve_single(o, d["rho0_packed"])
    assert abs(st["event_time"] - rst["event_time"]) <= 1e-12
    np.testing.assert_allclose(v, rv.reshape(-1), atol=1e-10)
    # batch form: per-trajectory event flags and times (ode_batch.rs:302-330)
    det = np.array([[0.0], [0.05], [3.0]], dtype=np.complex128)
    slot = d["payload"]["parameter_graph"]["slot_names"].index("delta")
    times, vals, width, tc, bst = api.solve_lindblad_batch_ode_py(
        plan, np.repeat(d["rho0_packed"].reshape(1, -1), 3, axis=0), 0.0, 5.0, 1e-10, 1e-8, 1e-3,
        parameter_slot_indices=[slot], parameter_batch=det, stop_event=ev)
    assert bst["event_count"] == sum(bst["event_triggered_by_trajectory"])
    assert times.size == 3


def test_expression_stop_event(golden):
    """A runtime-expression event t - 0.3 (the ragged-end-time form)."""
    d = golden("plan_two_level_td")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    ev = {"kind": "runtime_expression",
          "expression": {"instructions": [{"op": 4}, {"op": 1, "re": 0.3, "im": 0.0}, {"op": 6}], "scalar_only": True,
                         "output_is_tuple": False}}
    t, v, w, st = api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, 5.0, 1e-10, 1e-8, 1e-3, None, True, 100000,
                                            "expanded_sparse", "tsit5", "populations", None, "saveat", None, ev)
    assert st["event_triggered"]
    assert abs(st["event_time"] - 0.3) <= 1e-12
    assert abs(t[-1] - 0.3) <= 1e-12


def test_trajectory_error_messages_match_oracle(golden):
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=0.0, t1=1.0, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=None, save_start=True, maxiters=1,
                   solver="dopri5", output="populations", output_indices=None, output_when="saveat",
                   integral_weights=None, stop_event=None)
    with pytest.raises(oracle.OracleError) as ref:
        op.solve_single(o, d["rho0_packed"])
    with pytest.raises(ValueError) as got:
        api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, 1.0, 1e-10, 1e-8, 1e-3, None, True, 1, output="populations")
    assert str(got.value) == str(ref.value)
    with pytest.raises(ValueError, match=r"^trajectory 0: Stopped at x="):
        api.solve_lindblad_batch_ode_py(plan, np.repeat(d["rho0_packed"].reshape(1, -1), 2, axis=0), 0.0, 1.0, 1e-10,
                                        1e-8, 1e-3, maxiters=1)


def test_device_resident_batch_matches_host_batch(q1):
    torch = pytest.importorskip("torch")
    d, plan, _ = q1
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    params = _scan_params(d, 40, seed=11)
    slots = _slots(d)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), params.shape[0], axis=0)
    w = [(13, 1.0), (14, 1.0), (15, 1.0)]
    _, host_vals, _, _, _ = api.solve_lindblad_batch_ode_py(
        plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / gamma, solver="tsit5", output="excited_population",
        integral_weights=w, parameter_slot_indices=slots, parameter_batch=params)
    native = plan.native
    opts = native.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=None, save_start=True,
                          maxiters=100000, solver="tsit5", output="excited_population", output_indices=None,
                          output_when="final", integral_weights=w, stop_event=None)
    dev = torch.device("cuda:0")
    d_rho = torch.from_numpy(rho0).to(dev)
    d_par = torch.from_numpy(params.view(np.float64).reshape(-1)).to(dev)
    d_val = torch.zeros(params.shape[0], dtype=torch.float64, device=dev)
    d_st = torch.zeros(params.shape[0] * 6, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    native.solve_batch_device(opts, params.shape[0], d_rho.data_ptr(), slots, d_par.data_ptr(), 1, d_val.data_ptr(),
                              d_st.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_val.cpu().numpy(), np.asarray(host_vals))
    status = d_st.view(params.shape[0], 6)[:, 3].cpu().numpy() >> 32
    assert np.all(status == 0)


def test_mixed_form_keeps_the_trace(q1):
    """The mixed form renormalises the trace in double precision after every accepted step on a
    trace-preserving plan: the final populations sum to the initial trace to rounding (the
    single-precision-control variant, which does not renormalise, drifts by its rounding)."""
    d, plan, op = q1
    assert plan.native.trace_preserving
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    params = _scan_params(d, 64, seed=21)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), params.shape[0], axis=0)
    drift = {}
    for precision in ("mixed", "mixed_fp32_control"):
        _, pops, _, _, _ = api.solve_lindblad_batch_ode_py(
            plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / gamma, solver="tsit5", output="populations",
            parameter_slot_indices=_slots(d), parameter_batch=params, precision=precision)
        drift[precision] = float(np.max(np.abs(np.asarray(pops).reshape(-1, 16).sum(axis=1) - 1.0)))
    assert drift["mixed"] <= 1e-13, drift
    assert drift["mixed_fp32_control"] <= 1e-6, drift


def test_cost_ordered_queue_leaves_every_trajectory_unchanged(q1):
    """A batch larger than the launch's resident trajectory groups runs its queue longest-first by a
    cost estimate; every trajectory's values and statistics are exactly those of the same points
    solved in small single-wave batches (index order)."""
    d, plan, _ = q1
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    params = _scan_params(d, 3000, seed=17)
    slots = _slots(d)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), params.shape[0], axis=0)
    kw = dict(solver="tsit5", output="excited_population", integral_weights=[(13, 1.0), (14, 1.0), (15, 1.0)],
              parameter_slot_indices=slots, precision="mixed_fp32_control")
    _, whole, _, _, st = api.solve_lindblad_batch_ode_py(plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / gamma,
                                                         parameter_batch=params, **kw)
    assert plan.native.launches() == 5  # the queue ordering's four kernels and the integrator
    parts, acc = [], 0
    for lo in range(0, 3000, 500):
        _, v, _, _, s_ = api.solve_lindblad_batch_ode_py(plan, rho0[lo:lo + 500], t0, t1, 1e-11, 1e-8, 1e-3 / gamma,
                                                         parameter_batch=params[lo:lo + 500], **kw)
        assert plan.native.launches() == 1
        parts.append(np.asarray(v))
        acc += s_["accepted_steps"]
    np.testing.assert_array_equal(np.asarray(whole), np.concatenate(parts))
    assert st["accepted_steps"] == acc
