"""GPU parity of the large-system path (n > 45: 256 threads per trajectory, stage buffers in a
per-trajectory slice of device memory) on the 76-state rotational-cooling system: X J=0-3 + B
J'=1 F1'=1/2, 3/2 with R(0) and P(2) lasers whose polarisations switch as 1 MHz square waves.

Tolerances: the FP64 RHS within 1e-10 relative of the reference's Python RHS (pure arithmetic).
The square-wave drive makes the RHS discontinuous in time: at each switch the controller rejects
and retries, and rounding-level differences in h decide where the step past the jump lands, so
whole solves agree to the solver's tolerance (rtol 1e-8) rather than to rounding -- 1e-7
absolute on populations for both forms (the mixed form's headline bar is 1e-6), and 5e-6
relative on time integrals, which are trapezoids over the accepted steps and collect the
landing error of every jump (any change of the gather's summation order moves one of these
integrals by 1.4e-6 relative; with the switching frequency at zero the same system agrees with
the oracle to 1e-9, test_rc76_smooth_drive_matches_oracle_to_rounding).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api
from centrex_tlf_gb300.native import NativePlan

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rc(golden):
    d = golden("plan_rc_76")
    return d, api.prepare_lindblad_problem_py(d["payload"]), oracle.OraclePlan(d["payload"])


def _slots(d, names):
    return [d["payload"]["parameter_graph"]["slot_names"].index(s) for s in names]


def _params(d, count, seed):
    """Per-laser Rabi rate U[0.5, 3] Γ and detuning N(0, 0.5 Γ), seeded."""
    g = d["gamma"]
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(0.5, 3.0, count) * g, rng.uniform(0.5, 3.0, count) * g,
                     rng.normal(0.0, 0.5, count) * g, rng.normal(0.0, 0.5, count) * g], axis=1).astype(np.complex128)


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-10), ("mixed", 2e-5)])
def test_rc76_rhs_matches_python_reference(golden, precision, rtol):
    plan = NativePlan(golden("plan_rc_76")["payload"])
    for case in golden("rhs_rc_76")["cases"]:
        dy = plan.rhs(case["packed"], case["t"], case["override_slots"], case["override_values"], precision=precision)[0]
        ref = case["structured"]
        scale = float(np.max(np.abs(ref)))
        assert np.max(np.abs(dy - ref)) <= rtol * scale


@pytest.mark.parametrize("solver,precision,tol", [("tsit5", "fp64", 1e-7), ("dopri5", "fp64", 1e-7),
                                                  ("tsit5", "mixed", 1e-6)])
def test_rc76_scan_matches_oracle(rc, solver, precision, tol):
    """Final populations of a seeded four-point scan over 20/Γ (40 square-wave half periods)."""
    d, plan, op = rc
    g = d["gamma"]
    t1 = 20.0 / g
    slots = _slots(d, ("Ω0", "Ω1", "δ0", "δ1"))
    params = _params(d, 4, seed=7)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), params.shape[0], axis=0)
    _, pops, width, tc, st = api.solve_lindblad_batch_ode_py(
        plan, rho0, 0.0, t1, 1e-11, 1e-8, 1e-3 / g, solver=solver, output="populations",
        parameter_slot_indices=slots, parameter_batch=params, precision=precision)
    o = op.options(t0=0.0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([t1]), save_start=False,
                   maxiters=100000, solver=solver, output="populations", output_indices=None, output_when="final",
                   integral_weights=None, stop_event=None)
    ref, _, rst = op.solve_batch(o, rho0, slots, params)
    pops = np.asarray(pops).reshape(params.shape[0], 76)
    err = float(np.max(np.abs(pops - ref.reshape(params.shape[0], 76))))
    assert err <= tol, f"max population error {err:.3e}"
    np.testing.assert_allclose(pops.sum(axis=1), 1.0, atol=1e-9)
    assert abs(st["accepted_steps"] - int(rst["accepted_steps"].sum())) <= 0.02 * int(rst["accepted_steps"].sum()) + 4


def test_rc76_ragged_end_times_by_stop_event(rc):
    """Uneven end times per trajectory: a scanned t_end feeds a `Time() - t_end` stop event, and the
    excited-population integral stops there (the reference's route for ragged batches)."""
    d, plan, op = rc
    g = d["gamma"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = _slots(d, ("Ω0", "Ω1", "δ0", "δ1", "t_end"))
    base = _params(d, 3, seed=11)
    t_end = np.array([6.0, 11.0, 15.5]) / g
    params = np.concatenate([base, t_end.reshape(-1, 1).astype(np.complex128)], axis=1)
    ev = {"kind": "runtime_expression",
          "expression": {"instructions": [{"op": 4}, {"op": 2, "index": names.index("t_end")}, {"op": 6}],
                         "scalar_only": True, "output_is_tuple": False}}
    w = [(i, 1.0) for i in d["excited_indices"]]
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), 3, axis=0)
    _, v, _, _, st = api.solve_lindblad_batch_ode_py(
        plan, rho0, 0.0, 20.0 / g, 1e-11, 1e-8, 1e-3 / g, solver="tsit5", output="excited_population",
        integral_weights=w, parameter_slot_indices=slots, parameter_batch=params, stop_event=ev)
    assert list(st["event_triggered_by_trajectory"]) == [True, True, True]
    np.testing.assert_allclose(np.asarray(st["event_times"], dtype=float), t_end, rtol=1e-12)
    o = op.options(t0=0.0, t1=20.0 / g, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None, save_start=True,
                   maxiters=100000, solver="tsit5", output="excited_population", output_indices=None,
                   output_when="final", integral_weights=w, stop_event=ev)
    ref, _, _ = op.solve_batch(o, rho0, slots, params)
    np.testing.assert_allclose(np.asarray(v).reshape(-1), ref.reshape(-1), rtol=5e-6, atol=0.0)


@pytest.mark.parametrize("solver", ["tsit5", "dopri5"])
def test_rc76_smooth_drive_matches_oracle_to_rounding(rc, solver):
    """With the switching frequency scanned to zero the polarisations hold still (x for both
    lasers), the RHS is smooth, and FP64 solves agree with the oracle to 1e-9 on populations."""
    d, plan, op = rc
    g = d["gamma"]
    t1 = 20.0 / g
    slots = _slots(d, ("Ω0", "Ω1", "δ0", "δ1", "omega_pol"))
    base = _params(d, 4, seed=5)
    params = np.concatenate([base, np.zeros((4, 1), dtype=np.complex128)], axis=1)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), 4, axis=0)
    _, pops, _, _, st = api.solve_lindblad_batch_ode_py(
        plan, rho0, 0.0, t1, 1e-11, 1e-8, 1e-3 / g, solver=solver, output="populations",
        parameter_slot_indices=slots, parameter_batch=params)
    o = op.options(t0=0.0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([t1]), save_start=False,
                   maxiters=100000, solver=solver, output="populations", output_indices=None, output_when="final",
                   integral_weights=None, stop_event=None)
    ref, _, rst = op.solve_batch(o, rho0, slots, params)
    err = float(np.max(np.abs(np.asarray(pops).reshape(4, 76) - ref.reshape(4, 76))))
    assert err <= 1e-9, f"max population error {err:.3e}"
    assert abs(st["accepted_steps"] - int(rst["accepted_steps"].sum())) <= 0.02 * int(rst["accepted_steps"].sum()) + 4
