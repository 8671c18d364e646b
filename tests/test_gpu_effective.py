"""GPU parity of the interpolated effective-Hamiltonian path (prepare_effective_lindblad_plan_py,
solve_effective_lindblad_py, solve_effective_lindblad_batch_py, debug_effective_lindblad_rhs_py;
rust/src/effective_lindblad) against the reference's superoperators and the CPU oracle.

Tolerances: the RHS within 1e-12 relative of the values from the reference's node superoperators
(pure arithmetic); solves within 1e-9 of the oracle (the same Dopri5/Tsit5 steps, rounding-level
differences), step counts within 2 %; error messages identical.
"""

from __future__ import annotations

import copy

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eff(golden):
    d = golden("plan_eff_r0")
    return d, api.prepare_effective_lindblad_plan_py(d["plan"]), oracle.EffectiveOraclePlan(d["plan"])


def test_effective_rhs_matches_reference_superoperators(eff):
    d, plan, _ = eff
    for c in d["rhs_cases"]:
        dy = plan.native.rhs(c["y"], c["t"], [0, 1], np.array([c["base_rabi"], c["base_detuning"]], dtype=complex))[0]
        np.testing.assert_allclose(dy, c["dy"], rtol=1e-12, atol=1e-12 * np.max(np.abs(c["dy"])))
    # the debug call reads the base values: field, Rabi rate and detuning programs at t, the interval
    c = d["rhs_cases"][2]
    info = api.debug_effective_lindblad_rhs_py(plan, c["y"], c["t"])
    assert info["field_val"] == pytest.approx(150.0 + 40.0 * np.sin(2 * np.pi * 1e5 * c["t"]), rel=1e-14)
    assert info["rabi_val"] == pytest.approx(1.0e7 * np.exp(-(c["t"] - 2.5e-6) ** 2 / (2 * (1e-6) ** 2)), rel=1e-14)
    assert info["detuning_val"] == pytest.approx(2.0e11 * (c["t"] - 2.5e-6), rel=1e-12)
    assert info["last_interval"] == (1 if info["field_val"] > 150.0 else 0)
    assert not info["has_nan"] and info["dy_max"] == pytest.approx(np.max(np.abs(info["dy"])))


@pytest.mark.parametrize("solver", ["tsit5", "dopri5"])
def test_effective_single_solves_match_oracle(eff, solver):
    d, plan, op = eff
    t0, t1 = d["t_span"]
    saveat = np.linspace(t0, t1, 11)
    for output, kw in (("populations", {}), ("full", {}), ("selected", {"output_indices": [(0, 0), (0, 7), (7, 0)]}),
                       ("photon_integral", {"integral_weights": [(i * 11, 1.0) for i in (7, 8, 9)]})):
        sv = None if output == "photon_integral" else saveat
        times, values, width = api.solve_effective_lindblad_py(plan, d["y0"], t0, t1, 1e-9, 1e-7, 1e-10, sv, True, 100000,
                                                               solver, output, kw.get("output_indices"),
                                                               kw.get("integral_weights"))
        o = op.options(t0=t0, t1=t1, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=sv, save_start=True, maxiters=100000,
                       solver=solver, output=output, output_indices=kw.get("output_indices"),
                       integral_weights=kw.get("integral_weights"), output_when="final")
        rt, rv, _ = op.solve_single(o, d["y0"])
        np.testing.assert_array_equal(times, rt)
        assert width == o.width
        ref = np.asarray(rv).reshape(-1)
        scale = max(float(np.max(np.abs(ref))), 1e-300)
        np.testing.assert_allclose(np.asarray(values).reshape(-1), ref, rtol=0, atol=1e-9 * scale, err_msg=output)


def test_effective_batch_matches_oracle(eff):
    d, plan, op = eff
    t0, t1 = d["t_span"]
    saveat = np.linspace(t0, t1, 6)
    rng = np.random.default_rng(4)
    pb = np.stack([rng.uniform(0.3e7, 2.0e7, 8), rng.uniform(-5e6, 5e6, 8)], axis=1)
    times, values, width, tc, st = api.solve_effective_lindblad_batch_py(
        plan, d["y0"], t0, t1, 1e-9, 1e-7, 1e-10, saveat, True, 100000, "tsit5", "populations", None, None, [0, 1], pb, 8)
    assert (width, tc, st["trajectory_count"]) == (10, 6, 8)
    np.testing.assert_array_equal(times, saveat)
    o = op.options(t0=t0, t1=t1, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=saveat, save_start=True, maxiters=100000,
                   solver="tsit5", output="populations", output_indices=None, integral_weights=None)
    ref, _, rst = op.solve_batch(o, d["y0"], [0, 1], pb.astype(complex), time_count=6)
    np.testing.assert_allclose(np.asarray(values).reshape(ref.shape), ref, rtol=0, atol=1e-9)
    assert abs(st["accepted_steps"] - int(rst["accepted_steps"].sum())) <= 0.02 * int(rst["accepted_steps"].sum())
    # the trajectories really differ, and each one's trace stays 1
    pops = np.asarray(values).reshape(8, 6, 10)
    assert np.ptp(pops[:, -1, 7:].sum(axis=1)) > 1e-4
    np.testing.assert_allclose(pops.sum(axis=2), 1.0, atol=1e-7)


def test_effective_time_independent_detuning_is_frozen(golden):
    """δ0 = detuning is fixed at plan creation (effective_lindblad/plan.rs detect_constant_slot):
    a batch over `detuning` gives one answer, the oracle's."""
    d = golden("plan_eff_r0_static")
    plan = api.prepare_effective_lindblad_plan_py(d["plan"])
    op = oracle.EffectiveOraclePlan(d["plan"])
    pb = np.array([[1.0e7, -4e6], [1.0e7, 0.0], [1.0e7, 6e6]])
    _, values, _, _, _ = api.solve_effective_lindblad_batch_py(
        plan, d["y0"], 0.0, 5e-6, 1e-9, 1e-7, 1e-10, None, True, 100000, "tsit5", "photon_integral", None,
        [(i * 11, 1.0) for i in (7, 8, 9)], [0, 1], pb, 3)
    v = np.asarray(values)
    assert v[0] == v[1] == v[2]
    o = op.options(t0=0.0, t1=5e-6, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=None, save_start=True, maxiters=100000,
                   solver="tsit5", output="photon_integral", output_indices=None,
                   integral_weights=[(i * 11, 1.0) for i in (7, 8, 9)], output_when="final")
    ref, _, _ = op.solve_batch(o, d["y0"], [0, 1], pb.astype(complex))
    np.testing.assert_allclose(v, ref.reshape(-1), rtol=1e-9)


def test_effective_field_outside_the_grid_fails_like_the_reference(golden):
    """A grid that ends at 160 V/cm while the field program reaches 190: the reference's message
    ("field coordinate 1.6xxxxxe2 is above the operator grid maximum 1.600000e2"), from the
    solve and from the debug RHS, identical to the oracle's."""
    d = golden("plan_eff_r0")
    pd = copy.deepcopy(d["plan"])
    pd["field_grid"] = np.array([100.0, 130.0, 160.0])
    plan = api.prepare_effective_lindblad_plan_py(pd)
    op = oracle.EffectiveOraclePlan(pd)
    o = op.options(t0=0.0, t1=5e-6, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=np.array([5e-6]), save_start=False,
                   maxiters=100000, solver="tsit5", output="populations", output_indices=None, integral_weights=None)
    with pytest.raises(oracle.OracleError) as ref:
        op.solve_batch(o, d["y0"], [0], np.array([[1e7]], dtype=complex))
    with pytest.raises(ValueError) as got:
        api.solve_effective_lindblad_batch_py(plan, d["y0"], 0.0, 5e-6, 1e-9, 1e-7, 1e-10, np.array([5e-6]), False, 100000,
                                              "tsit5", "populations", None, None, [0], np.array([[1e7]]), 1)
    assert str(got.value) == str(ref.value)
    assert "is above the operator grid maximum 1.600000e2" in str(got.value)
    t_hi = 0.25e-5  # Ez = 190
    with pytest.raises(ValueError, match=r"^field coordinate 1\.900000e2 is above the operator grid maximum 1\.600000e2$"):
        api.debug_effective_lindblad_rhs_py(plan, d["y0"], t_hi)
