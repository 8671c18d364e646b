"""GPU parity of the fixed-step solvers (fixed_dopri5, fixed_rk2, fixed_rk4; rust/src/ode/fixed.rs)
against the reference's recorded fixed-step runs and the CPU oracle.

A fixed-step run has no controller feedback: the step sequence is the same on both sides, so the
GPU differs from the oracle by rounding alone (fused multiply-adds, summation order).  Tolerance:
1e-12 relative on integrals and 1e-12 absolute on populations.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu

FIXED_CASES = ["fixed_dopri5_dt5e-2", "fixed_dopri5_dt1e-3", "fixed_rk4_dt5e-2", "fixed_rk4_dt2e-3",
               "fixed_rk2_dt1e-2", "fixed_rk2_dt5e-4"]


def _slot(d, name):
    return d["payload"]["parameter_graph"]["slot_names"].index(name)


@pytest.mark.parametrize("label", FIXED_CASES)
def test_fixed_step_known_answers(golden, label):
    """The reference's fixed-step benchmark (two-level, Omega 0.8, photon integral over [0, 0.8]):
    single-run and 201-point-grid step counts, and the photon integral against the reference's
    value rebuilt from its recorded abs/rel errors against the adaptive run."""
    d = golden("plan_two_level")
    kat = golden("kat_fixed_step")
    case = kat["cases"][label]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    t0, t1 = kat["t_span"]
    slots = [_slot(d, "Omega"), _slot(d, "delta")]
    _, v, _, _, st = api.solve_lindblad_batch_ode_py(
        plan, d["rho0_packed"].reshape(1, -1), t0, t1, kat["abstol"], kat["reltol"], case["dt"], solver=case["solver"],
        output="photon_integral", integral_weights=[(1, 0.3)], parameter_slot_indices=slots,
        parameter_batch=np.array([[kat["omega"], kat["delta"]]], dtype=complex))
    assert (st["accepted_steps"], st["rejected_steps"], st["rhs_calls"]) == (
        case["single_accepted_steps"], 0, case["single_rhs_calls"])
    _, va, _, _, _ = api.solve_lindblad_batch_ode_py(
        plan, d["rho0_packed"].reshape(1, -1), t0, t1, kat["abstol"], kat["reltol"], 1e-3, solver="dopri5",
        output="photon_integral", integral_weights=[(1, 0.3)], parameter_slot_indices=slots,
        parameter_batch=np.array([[kat["omega"], kat["delta"]]], dtype=complex))
    ref_adaptive = case["abs_error_vs_adaptive"] / case["rel_error_vs_adaptive"]
    ref_fixed = ref_adaptive + np.sign(v[0] - va[0]) * case["abs_error_vs_adaptive"]
    assert abs(v[0] - ref_fixed) <= 1e-12 * ref_fixed
    # the grid form: Omega fixed, 201 detunings, last axis fastest
    axes = np.concatenate([[kat["omega"]], kat["grid_detuning"]]).astype(complex)
    _, gv, _, tc, gst = api.solve_lindblad_grid_ode_py(
        plan, d["rho0_packed"], t0, t1, kat["abstol"], kat["reltol"], case["dt"], slots, axes, [1, 201],
        solver=case["solver"], output="photon_integral", integral_weights=[(1, 0.3)])
    assert tc == 1
    assert (gst["accepted_steps"], gst["rhs_calls"]) == (case["grid_accepted_steps"], case["grid_rhs_calls"])
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=t0, t1=t1, abstol=kat["abstol"], reltol=kat["reltol"], dt=case["dt"], saveat=None,
                   save_start=True, maxiters=100000, solver=case["solver"], output="photon_integral",
                   output_indices=None, output_when="final", integral_weights=[(1, 0.3)], stop_event=None)
    params = np.stack([np.full(201, kat["omega"]), kat["grid_detuning"]], axis=1).astype(complex)
    ref, _, _ = op.solve_batch(o, d["rho0_packed"], slots, params)
    np.testing.assert_allclose(np.asarray(gv).reshape(-1), ref.reshape(-1), rtol=1e-12)


@pytest.mark.parametrize("solver", ["fixed_dopri5", "fixed_rk4", "fixed_rk2"])
def test_q1_fixed_step_saveat_matches_oracle(golden, solver):
    """The 16-state Gaussian-pulse system (time-dependent coefficients at every stage time),
    saveat populations and the excited-population integral, on a few scan points."""
    d = golden("plan_q1_16")
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    op = oracle.OraclePlan(d["payload"])
    slots = [_slot(d, s) for s in ("rabi", "detuning", "theta")]
    params = np.array([[gamma, 0.0, 0.3], [3.0 * gamma, -2.0 * gamma, 1.1], [0.3 * gamma, 4.0 * gamma, 2.5]], dtype=complex)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), params.shape[0], axis=0)
    dt = (0.05 if solver == "fixed_rk2" else 0.2) / gamma
    saveat = np.linspace(t0, t1, 13)
    times, pops, _, tc, st = api.solve_lindblad_batch_ode_py(
        plan, rho0, t0, t1, 1e-11, 1e-8, dt, saveat=saveat, solver=solver, output="populations",
        output_when="saveat", parameter_slot_indices=slots, parameter_batch=params)
    o = op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=dt, saveat=saveat, save_start=True, maxiters=100000,
                   solver=solver, output="populations", output_indices=None, output_when="saveat",
                   integral_weights=None, stop_event=None)
    ref, rt, rst = op.solve_batch(o, rho0, slots, params, time_count=saveat.size)
    assert tc == saveat.size
    np.testing.assert_array_equal(np.asarray(times), rt)
    np.testing.assert_allclose(np.asarray(pops).reshape(ref.shape), ref, rtol=0, atol=1e-12)
    assert st["accepted_steps"] == int(rst["accepted_steps"].sum())
    assert st["rhs_calls"] == int(rst["rhs_calls"].sum())
    w = [(13, 1.0), (14, 1.0), (15, 1.0)]
    _, integ, _, _, _ = api.solve_lindblad_batch_ode_py(
        plan, rho0, t0, t1, 1e-11, 1e-8, dt, solver=solver, output="excited_population", integral_weights=w,
        parameter_slot_indices=slots, parameter_batch=params)
    o = op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=dt, saveat=None, save_start=True, maxiters=100000,
                   solver=solver, output="excited_population", output_indices=None, output_when="final",
                   integral_weights=w, stop_event=None)
    ref, _, _ = op.solve_batch(o, rho0, slots, params)
    np.testing.assert_allclose(np.asarray(integ).reshape(-1), ref.reshape(-1), rtol=1e-12)


def test_fixed_step_event_and_errors(golden):
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    op = oracle.OraclePlan(d["payload"])
    ev = {"kind": "population", "indices": [1], "threshold": 0.05}
    t, v, w, st = api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, 5.0, 1e-10, 1e-8, 0.01, None, True, 100000,
                                            "expanded_sparse", "fixed_rk4", "populations", None, "saveat", None, ev)
    o = op.options(t0=0.0, t1=5.0, abstol=1e-10, reltol=1e-8, dt=0.01, saveat=None, save_start=True, maxiters=100000,
                   solver="fixed_rk4", output="populations", output_indices=None, output_when="saveat",
                   integral_weights=None, stop_event=ev)
    rt, rv, rst = op.solve_single(o, d["rho0_packed"])
    assert st["event_triggered"] and rst["event_triggered"]
    assert st["event_time"] == rst["event_time"]
    np.testing.assert_array_equal(t, rt)
    np.testing.assert_allclose(v.reshape(rv.shape), rv, atol=1e-13)
    with pytest.raises(ValueError, match="^fixed-step solvers require positive finite dt$"):
        api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, 1.0, 1e-10, 1e-8, 0.0, solver="fixed_rk2")
    with pytest.raises(ValueError, match=r"^Stopped at x=0\.2\. Need more than 2 steps\.$"):
        api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, 1.0, 1e-10, 1e-8, 0.1, None, True, 2,
                                  solver="fixed_dopri5")
    with pytest.raises(NotImplementedError, match="adaptive solvers"):
        api.solve_lindblad_batch_ode_py(plan, d["rho0_packed"].reshape(1, -1), 0.0, 1.0, 1e-10, 1e-8, 0.1,
                                        solver="fixed_rk4", precision="mixed")
