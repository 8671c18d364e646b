"""GPU checks of the launch shapes (obe_plan_set_shape / obe_plan_autotune).

Every compiled width that holds a system solves it; a width changes the gather's summation order
and so the rounding, not the result: FP64 populations within 1e-9 of the oracle at every shape
(the same bar as the default shape), the mixed form within its 1e-6 bar of FP64.  The autotuner
returns its measured candidates, keeps the fastest and leaves the plan solving correctly.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu


def _q1_batch(d, count, seed):
    g = d["gamma"]
    rng = np.random.default_rng(seed)
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [names.index(s) for s in ("rabi", "detuning", "theta")]
    params = np.stack([g * 10 ** rng.uniform(-1.0, 1.0, count), rng.uniform(-5.0, 5.0, count) * g,
                       rng.uniform(0.0, np.pi, count)], axis=1).astype(np.complex128)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), count, axis=0)
    return slots, params, rho0


def _final_pops(plan, d, rho0, slots, params, precision="fp64", solver="tsit5", t1=None):
    g = d["gamma"]
    t1 = d["t_span"][1] if t1 is None else t1
    _, v, _, _, st = api.solve_lindblad_batch_ode_py(
        plan, rho0, 0.0, t1, 1e-11, 1e-8, 1e-3 / g, solver=solver, output="populations",
        parameter_slot_indices=slots, parameter_batch=params, precision=precision)
    n = d["payload"]["n_states"]
    return np.asarray(v).reshape(-1, n), st


def _oracle_pops(d, rho0, slots, params, solver="tsit5", t1=None):
    g = d["gamma"]
    t1 = d["t_span"][1] if t1 is None else t1
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=0.0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([t1]), save_start=False,
                   maxiters=100000, solver=solver, output="populations", output_indices=None, output_when="final",
                   integral_weights=None, stop_event=None)
    ref, _, _ = op.solve_batch(o, rho0, slots, params)
    return ref.reshape(rho0.shape[0], -1)


def test_every_16_state_shape_matches_oracle(golden):
    d = golden("plan_q1_16")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    slots, params, rho0 = _q1_batch(d, 24, seed=8)
    ref = _oracle_pops(d, rho0, slots, params)
    try:
        for tpt, gpb in ((32, 0), (32, 1), (64, 0), (64, 2), (128, 0), (128, 1)):
            plan.native.set_shape(tpt, gpb)
            assert plan.native.shape() == (tpt, gpb)
            pops, _ = _final_pops(plan, d, rho0, slots, params)
            err = float(np.max(np.abs(pops - ref)))
            assert err <= 1e-9, f"shape ({tpt}, {gpb}): max population error {err:.3e}"
            mixed, _ = _final_pops(plan, d, rho0, slots, params, precision="mixed")
            assert float(np.max(np.abs(mixed - pops))) <= 1e-6
    finally:
        plan.native.set_shape(0, 0)


def test_autotune_keeps_its_fastest_candidate(golden):
    d = golden("plan_q1_16")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    slots, params, rho0 = _q1_batch(d, 512, seed=9)
    g = d["gamma"]
    try:
        cands = api.autotune_lindblad_batch_py(
            plan, rho0, 0.0, d["t_span"][1], 1e-11, 1e-8, 1e-3 / g, probe_steps=24, solver="tsit5",
            output="excited_population", integral_weights=[(13, 1.0), (14, 1.0), (15, 1.0)],
            parameter_slot_indices=slots, parameter_batch=params, precision="mixed")
        assert {c["threads_per_trajectory"] for c in cands} == {32, 64, 128}
        assert all(c["probe_ms"] > 0.0 for c in cands)
        best = cands[0]
        assert best["probe_ms"] == min(c["probe_ms"] for c in cands)
        assert plan.native.shape() == (best["threads_per_trajectory"], best["trajectories_per_cta"])
        # the tuned plan still solves correctly (FP64 against the oracle on a few points)
        pops, _ = _final_pops(plan, d, rho0[:8], slots, params[:8])
        assert float(np.max(np.abs(pops - _oracle_pops(d, rho0[:8], slots, params[:8])))) <= 1e-9
    finally:
        plan.native.set_shape(0, 0)


@pytest.mark.parametrize("wide", [False, True])
def test_76_state_wide_shape_matches_oracle(golden, monkeypatch, wide):
    """256 and 512 threads per trajectory on the 76-state system, smooth drive (switching
    frequency 0): the tight shapes (24 and 12 elements per thread) and, with OBE_EPT_WIDE, the
    widest ones (32 and 16), which systems of 79-90 states run."""
    if wide:
        monkeypatch.setenv("OBE_EPT_WIDE", "1")
    d = golden("plan_rc_76")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    g = d["gamma"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [names.index(s) for s in ("Ω0", "Ω1", "δ0", "δ1", "omega_pol")]
    rng = np.random.default_rng(5)
    params = np.stack([rng.uniform(0.5, 3.0, 3) * g, rng.uniform(0.5, 3.0, 3) * g, rng.normal(0.0, 0.5, 3) * g,
                       rng.normal(0.0, 0.5, 3) * g, np.zeros(3)], axis=1).astype(np.complex128)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), 3, axis=0)
    ref = _oracle_pops(d, rho0, slots, params, t1=20.0 / g)
    try:
        for tpt in (256, 512):
            plan.native.set_shape(tpt, 0)
            pops, _ = _final_pops(plan, d, rho0, slots, params, t1=20.0 / g)
            err = float(np.max(np.abs(pops - ref)))
            assert err <= 1e-9, f"{tpt} threads: max population error {err:.3e}"
    finally:
        plan.native.set_shape(0, 0)


def test_gradients_need_a_narrow_layout(golden):
    import torch

    from centrex_tlf_gb300.autograd import solve_batch_with_grad
    from centrex_tlf_gb300.native import NativePlan

    d = golden("plan_q1_16")
    plan = NativePlan(d["payload"])
    names = d["payload"]["parameter_graph"]["slot_names"]
    p = torch.tensor([[d["gamma"], 0.0]], dtype=torch.float64, device="cuda", requires_grad=True)
    plan.set_shape(512, 0)
    with pytest.raises(NotImplementedError, match="gradients need the plan at 256 threads per trajectory or fewer"):
        solve_batch_with_grad(plan, d["rho0_packed"], d["t_span"], p, [names.index("rabi"), names.index("detuning")],
                              dt=1e-3 / d["gamma"], integral_weights=[(13, 1.0)])
    plan.set_shape(0, 0)
    j = solve_batch_with_grad(plan, d["rho0_packed"], d["t_span"], p, [names.index("rabi"), names.index("detuning")],
                              dt=1e-3 / d["gamma"], integral_weights=[(13, 1.0)])
    j.sum().backward()
    assert torch.isfinite(p.grad).all()
