"""The oracle on the interpolated effective-Hamiltonian path (rust/src/effective_lindblad),
pinned to the reference's own superoperators.

tests/golden/plan_eff_r0.json holds the payload the reference's prepare_effective_lindblad_rust_plan
builds for an R(0) F1'=1/2 F'=1 compact model on a three-point field grid (captured at its native
boundary) and RHS values computed from the reference's node superoperators
(effective_hamiltonian/_superoperators.py) -- at the middle node exactly, between the nodes
through their linear interpolation, which is what the payload's `linear` coefficients encode.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle


@pytest.fixture(scope="module")
def eff(golden):
    d = golden("plan_eff_r0")
    return d, oracle.EffectiveOraclePlan(d["plan"])


def test_effective_rhs_matches_reference_superoperators(eff):
    d, op = eff
    assert op.N == 2 * op.n * op.n == 200
    for c in d["rhs_cases"]:
        dy = op.rhs(c["y"], c["t"], [0, 1], np.array([c["base_rabi"], c["base_detuning"]], dtype=complex))
        np.testing.assert_allclose(dy, c["dy"], rtol=1e-12, atol=1e-12 * np.max(np.abs(c["dy"])))


def test_time_independent_detuning_program_is_frozen_at_its_base_value(golden, eff):
    """effective_lindblad/plan.rs detect_constant_slot: with δ0 = detuning (no time), the plan
    fixes δ at the base value when it is built, so a per-trajectory override of `detuning` does
    not reach the RHS; with a time-dependent δ0 it does."""
    d, op = eff
    static = oracle.EffectiveOraclePlan(golden("plan_eff_r0_static")["plan"])
    c = d["rhs_cases"][1]
    base = static.rhs(c["y"], c["t"], [0], np.array([c["base_rabi"]], dtype=complex))
    moved = static.rhs(c["y"], c["t"], [0, 1], np.array([c["base_rabi"], 3.0e6], dtype=complex))
    np.testing.assert_array_equal(base, moved)
    a = op.rhs(c["y"], c["t"], [0, 1], np.array([c["base_rabi"], 0.0], dtype=complex))
    b = op.rhs(c["y"], c["t"], [0, 1], np.array([c["base_rabi"], 3.0e6], dtype=complex))
    assert np.max(np.abs(a - b)) > 0


def test_effective_solve_conserves_trace(eff):
    d, op = eff
    t0, t1 = d["t_span"]
    saveat = np.linspace(t0, t1, 6)
    o = op.options(t0=t0, t1=t1, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=saveat, save_start=True, maxiters=100000,
                   solver="tsit5", output="populations", output_indices=None, integral_weights=None)
    times, pops, st = op.solve_single(o, d["y0"])
    np.testing.assert_array_equal(times, saveat)
    np.testing.assert_allclose(pops.sum(axis=1), 1.0, atol=1e-7)
    assert pops[0, d["ground_main"]] == 1.0 and pops[-1, d["ground_main"]] < 1.0
    assert st["accepted_steps"] > 10
