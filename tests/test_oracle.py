"""Pin the CPU oracle (oracle/obe_oracle.c) before any GPU result is compared with it.

Anchors, all from the reference itself:
* the two-level known answer of its packed-RHS benchmark
  (benchmarks/expanded_sparse_packed_rhs_results/validation.csv:5-8, solve_timings.csv:2,
  grid_timings.csv:2);
* its Python FP64 RHS evaluators run on the same payloads (tests/golden/rhs_*.json, made by
  tests/golden/make_fixtures.py from centrex_tlf/lindblad/reference_dense.py:60-77);
* its SciPy RK45 solves (tests/golden/rk45_*.json, centrex_tlf/lindblad/solve.py:155-199);
* its error messages (rust/src/ode/dopri5.rs:167-231, common.rs:124-151).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

PLANS = ["two_level", "two_level_td", "chain3", "chain45", "q1_16"]


def _plan(golden, name):
    return oracle.OraclePlan(golden(f"plan_{name}")["payload"])


def _opts(plan, **kw):
    base = dict(
        t0=0.0, t1=1.0, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=None, save_start=True,
        maxiters=100000, solver="dopri5", output="populations", output_indices=None,
        output_when="final", integral_weights=None, stop_event=None,
    )
    base.update(kw)
    return plan.options(**base)


def test_two_level_known_answer(golden):
    d = golden("plan_two_level")
    kat = d["kat"]
    p = oracle.OraclePlan(d["payload"])
    o = _opts(p, t1=0.5, abstol=kat["abstol"], reltol=kat["reltol"], dt=kat["dt"],
              output="photon_integral", integral_weights=[(1, 0.3)])
    _, v, st = p.solve_single(o, d["rho0_packed"])
    assert st["accepted_steps"] == kat["accepted_steps"] == 10
    assert st["rejected_steps"] == kat["rejected_steps"] == 0
    assert st["rhs_calls"] == kat["rhs_calls"] == 61
    # bit-identical to the reference's split-input kernel run (validation.csv:7-8)
    assert v[-1, 0] == 0.0010681268919861524
    # and within 1.1e-11 relative of its recorded baseline value (validation.csv:5)
    assert abs(v[-1, 0] - kat["photon_integral"]) <= 2e-11 * kat["photon_integral"]


def test_two_level_grid_known_answer(golden):
    d = golden("plan_two_level")
    kat = d["kat"]
    p = oracle.OraclePlan(d["payload"])
    o = _opts(p, t1=0.5, abstol=kat["abstol"], reltol=kat["reltol"], dt=kat["dt"],
              output="photon_integral", integral_weights=[(1, 0.3)])
    det = d["kat_grid"]["detuning"]
    slot = p.slot_names.index("delta")
    vals, times, stats = p.solve_batch(o, d["rho0_packed"], [slot], det.reshape(-1, 1).astype(complex))
    assert int(stats["accepted_steps"].sum()) == d["kat_grid"]["accepted_steps"] == 252
    assert int(stats["rejected_steps"].sum()) == 0
    assert int(stats["rhs_calls"].sum()) == d["kat_grid"]["rhs_calls"] == 1537
    assert times[0] == 0.5
    # the photon line is symmetric in the detuning and peaks on resonance
    line = vals[:, 0, 0]
    assert int(np.argmax(line)) == 12
    np.testing.assert_allclose(line, line[::-1], rtol=1e-6)


@pytest.mark.parametrize("name", PLANS + ["rc_76", "r0_39"])
def test_rhs_matches_python_reference(golden, name):
    p = _plan(golden, name)
    for case in golden(f"rhs_{name}")["cases"]:
        dy = p.rhs(case["packed"], case["t"], case["override_slots"], case["override_values"])
        ref = case["structured"]
        scale = float(np.max(np.abs(ref)))
        np.testing.assert_allclose(dy, ref, rtol=1e-9, atol=1e-12 * scale)
        # the dense C rho C^dagger form agrees as well (test_rust_backend.py:568 tolerance)
        np.testing.assert_allclose(dy, case["reference"], rtol=1e-9, atol=1e-12 * scale)


def test_split_input_orders_agree(golden):
    p = _plan(golden, "chain45")
    for case in golden("rhs_chain45")["cases"]:
        a = p.rhs(case["packed"], case["t"], case["override_slots"], case["override_values"], use_split_input_rhs=True)
        b = p.rhs(case["packed"], case["t"], case["override_slots"], case["override_values"], use_split_input_rhs=False)
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-13 * np.max(np.abs(a)))


@pytest.mark.parametrize("name,solver", [("two_level", "dopri5"), ("two_level_td", "tsit5"), ("chain3", "dopri5")])
def test_trajectory_matches_scipy_rk45(golden, name, solver):
    d = golden(f"plan_{name}")
    rk = golden(f"rk45_{name}")
    p = oracle.OraclePlan(d["payload"])
    t0, t1 = d["t_span"]
    o = _opts(p, t0=t0, t1=t1, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=rk["t"], output="full",
              output_when="saveat", solver=solver)
    t, v, _ = p.solve_single(o, d["rho0_packed"])
    np.testing.assert_allclose(t, rk["t"], rtol=0, atol=1e-15)
    # Rust-vs-RK45 tolerance of the reference (test_rust_backend.py:2118-2149)
    np.testing.assert_allclose(v, rk["packed_y"], atol=5e-7, rtol=5e-6)


@pytest.mark.parametrize("case", ["nominal", "detuned"])
def test_q1_trajectory_matches_scipy_rk45(golden, case):
    d = golden("plan_q1_16")
    rk = golden("rk45_q1_16")[case]
    p = oracle.OraclePlan(d["payload"])
    t0, t1 = d["t_span"]
    gamma = d["gamma"]
    o = _opts(p, t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=rk["t"], output="full",
              output_when="saveat")
    t, v, st = p.solve_single(o, d["rho0_packed"], rk["override_slots"], rk["override_values"])
    np.testing.assert_allclose(v, rk["packed_y"], atol=5e-7, rtol=5e-6)
    trace = v[:, :16].sum(axis=1)
    np.testing.assert_allclose(trace, 1.0, atol=2e-6)
    assert st["accepted_steps"] > 50


def test_outputs_are_consistent_with_full_trajectory(golden):
    """populations / selected / final-only agree with the full trajectory
    (test_rust_backend.py:873-927 tolerances)."""
    d = golden("plan_q1_16")
    p = oracle.OraclePlan(d["payload"])
    gamma = d["gamma"]
    t1 = d["t_span"][1]
    common = dict(t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma)
    saveat = np.linspace(0.0, t1, 7)
    _, full, _ = p.solve_single(_opts(p, saveat=saveat, output="full", output_when="saveat", **common), d["rho0_packed"])
    _, pops, _ = p.solve_single(_opts(p, saveat=saveat, output="populations", output_when="saveat", **common), d["rho0_packed"])
    np.testing.assert_allclose(pops, full[:, :16], atol=1e-12, rtol=1e-10)
    pairs = [(0, 13), (14, 2), (5, 5)]
    _, sel, _ = p.solve_single(_opts(p, saveat=saveat, output="selected", output_indices=pairs, output_when="saveat", **common), d["rho0_packed"])
    from centrex_tlf_gb300._options import packed_upper_real_index

    r = packed_upper_real_index(16, 0, 13)
    np.testing.assert_allclose(sel[:, 0], full[:, r] + 1j * full[:, r + 1], atol=1e-12)
    r = packed_upper_real_index(16, 2, 14)
    np.testing.assert_allclose(sel[:, 1], full[:, r] - 1j * full[:, r + 1], atol=1e-12)
    np.testing.assert_allclose(sel[:, 2], full[:, 5], atol=1e-12)


def test_integral_trace_final_and_rate_agree(golden):
    """The integral trace ends at the final integral; the rate trace integrates to it
    (test_rust_backend.py:1615-1694)."""
    d = golden("plan_q1_16")
    p = oracle.OraclePlan(d["payload"])
    gamma = d["gamma"]
    t1 = d["t_span"][1]
    w = [(13, 1.0), (14, 1.0), (15, 1.0)]
    common = dict(t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, integral_weights=w, solver="tsit5")
    _, fin, st = p.solve_single(_opts(p, output="excited_population", output_when="final", **common), d["rho0_packed"])
    t, trace, st2 = p.solve_single(_opts(p, output="excited_population", output_when="saveat", **common), d["rho0_packed"])
    assert fin.shape == (1, 1)
    assert trace.shape[0] == st2["accepted_steps"] + 1
    assert trace[-1, 0] == fin[0, 0]
    saveat = np.linspace(0.0, t1, 2001)
    ts, rate, _ = p.solve_single(_opts(p, output="excited_population_rate", output_when="saveat", saveat=saveat, **common), d["rho0_packed"])
    approx = np.trapezoid(rate[:, 0], ts)
    assert abs(approx - fin[0, 0]) <= 1e-3 * abs(fin[0, 0])


def test_population_stop_event(golden):
    d = golden("plan_two_level")
    p = oracle.OraclePlan(d["payload"])
    ev = {"kind": "population", "indices": [1], "threshold": 0.05}
    o = _opts(p, t1=5.0, stop_event=ev, output="populations", output_when="final", saveat=np.array([5.0]), save_start=False)
    t, v, st = p.solve_single(o, d["rho0_packed"])
    assert st["event_triggered"]
    assert t[-1] == st["event_time"] < 5.0
    assert abs(v[-1, 1] - 0.05) < 1e-9


def test_error_messages(golden):
    d = golden("plan_two_level")
    p = oracle.OraclePlan(d["payload"])
    with pytest.raises(oracle.OracleError, match=r"^Stopped at x=0\.\d+\. Need more than 2 steps\.$"):
        p.solve_single(_opts(p, maxiters=1), d["rho0_packed"])
    with pytest.raises(oracle.OracleError, match="only forward integration"):
        p.solve_single(_opts(p, t0=1.0, t1=0.5), d["rho0_packed"])
    with pytest.raises(oracle.OracleError, match=r"saveat value 2 is outside \[0, 1\]"):
        p.solve_single(_opts(p, saveat=np.array([0.5, 2.0]), output_when="saveat"), d["rho0_packed"])
    with pytest.raises(oracle.OracleError, match="maxiters must be positive"):
        p.solve_single(_opts(p, maxiters=0), d["rho0_packed"])
    # batch: first failing trajectory index prefix (ode_batch.rs:309)
    det = np.array([[0.0], [0.1]], dtype=complex)
    with pytest.raises(oracle.OracleError, match=r"^trajectory 0: Stopped at x="):
        p.solve_batch(_opts(p, maxiters=1), d["rho0_packed"], [p.slot_names.index("delta")], det)


def _fixed_kat_solve(p, d, kat, case, grid=False):
    """One run of the reference's fixed-step benchmark configuration
    (benchmarks/bench_fixed_step_solvers.py:124-160) through the oracle."""
    o = _opts(p, t0=kat["t_span"][0], t1=kat["t_span"][1], abstol=kat["abstol"], reltol=kat["reltol"],
              dt=case["dt"], solver=case["solver"], output="photon_integral",
              integral_weights=[tuple(w) for w in kat["weights"]])
    slots = [p.slot_names.index("Omega"), p.slot_names.index("delta")]
    det = kat["grid_detuning"] if grid else np.array([kat["delta"]])
    params = np.stack([np.full(det.size, kat["omega"]), det], axis=1).astype(complex)
    vals, _, st = p.solve_batch(o, d["rho0_packed"], slots, params)
    return vals[:, 0, 0], st


@pytest.mark.parametrize("label", ["fixed_dopri5_dt5e-2", "fixed_dopri5_dt2p5e-2", "fixed_dopri5_dt1e-3",
                                   "fixed_rk4_dt5e-2", "fixed_rk4_dt2p5e-2", "fixed_rk4_dt1e-3", "fixed_rk4_dt2e-3",
                                   "fixed_rk2_dt1e-2", "fixed_rk2_dt5e-4"])
def test_fixed_step_known_answers(golden, label):
    """Step and RHS counts of the reference's fixed-step runs, single and on the 201-point
    detuning grid, and the photon-integral difference of each from the adaptive Dopri5 run
    (benchmarks/fixed_step_solver_results/fixed_step_solver_report.md, fixed_step_solver_validation.csv)."""
    d = golden("plan_two_level")
    kat = golden("kat_fixed_step")
    p = oracle.OraclePlan(d["payload"])
    ref, st_ref = _fixed_kat_solve(p, d, kat, kat["cases"]["adaptive_dopri5"])
    assert int(st_ref["accepted_steps"][0]) == kat["cases"]["adaptive_dopri5"]["single_accepted_steps"] == 15
    assert int(st_ref["rhs_calls"][0]) == kat["cases"]["adaptive_dopri5"]["single_rhs_calls"] == 91
    case = kat["cases"][label]
    v, st = _fixed_kat_solve(p, d, kat, case)
    assert int(st["accepted_steps"][0]) == case["single_accepted_steps"]
    assert int(st["rhs_calls"][0]) == case["single_rhs_calls"]
    assert int(st["rejected_steps"][0]) == 0
    diff = abs(v[0] - ref[0])
    assert abs(diff - case["abs_error_vs_adaptive"]) <= 1e-9 * case["abs_error_vs_adaptive"]
    assert abs(diff / abs(ref[0]) - case["rel_error_vs_adaptive"]) <= 1e-9 * case["rel_error_vs_adaptive"]
    # the reference's fixed-step value itself, rebuilt from its recorded abs and rel errors
    # (adaptive = abs / rel, fixed = adaptive -/+ abs): the oracle matches it to the last bits
    ref_adaptive = case["abs_error_vs_adaptive"] / case["rel_error_vs_adaptive"]
    ref_fixed = ref_adaptive + np.sign(v[0] - ref[0]) * case["abs_error_vs_adaptive"]
    assert abs(v[0] - ref_fixed) <= 5e-16 * abs(ref_fixed)
    _, stg = _fixed_kat_solve(p, d, kat, case, grid=True)
    assert int(stg["accepted_steps"].sum()) == case["grid_accepted_steps"]
    assert int(stg["rhs_calls"].sum()) == case["grid_rhs_calls"]


def test_adaptive_grid_known_answer_of_fixed_step_benchmark(golden):
    d = golden("plan_two_level")
    kat = golden("kat_fixed_step")
    p = oracle.OraclePlan(d["payload"])
    case = kat["cases"]["adaptive_dopri5"]
    _, st = _fixed_kat_solve(p, d, kat, case, grid=True)
    assert int(st["accepted_steps"].sum()) == case["grid_accepted_steps"] == 3845
    assert int(st["rhs_calls"].sum()) == case["grid_rhs_calls"] == 23271


def test_fixed_step_saveat_and_errors(golden):
    d = golden("plan_two_level")
    p = oracle.OraclePlan(d["payload"])
    # steps shorten to land on saveat times (fixed.rs:16-26): 0.1 steps with saves at 0.25 and 0.5
    saveat = np.array([0.0, 0.25, 0.5])
    t, v, st = p.solve_single(_opts(p, t1=0.5, dt=0.1, solver="fixed_rk4", output="populations",
                                    output_when="saveat", saveat=saveat), d["rho0_packed"])
    np.testing.assert_array_equal(t, saveat)
    assert st["accepted_steps"] == 6  # 0.1 0.2 0.25 0.35 0.45 0.5
    full = _opts(p, t1=0.5, dt=0.1, solver="fixed_rk4", output="populations", output_when="saveat")
    t2, v2, _ = p.solve_single(full, d["rho0_packed"])
    np.testing.assert_allclose(t2, [0.0, 0.1, 0.2, 0.30000000000000004, 0.4, 0.5])
    with pytest.raises(oracle.OracleError, match="^fixed-step solvers require positive finite dt$"):
        p.solve_single(_opts(p, dt=0.0, solver="fixed_rk2"), d["rho0_packed"])
    with pytest.raises(oracle.OracleError, match=r"^Stopped at x=0\.2\. Need more than 2 steps\.$"):
        p.solve_single(_opts(p, dt=0.1, maxiters=2, solver="fixed_dopri5"), d["rho0_packed"])


def test_r2_38_state_known_answer(golden):
    """The reference's heavy known answer: its Rust solve of the 38-state R(2) benchmark system
    (benchmarks/expanded_sparse_static_dynamic_results/solve_timings.csv:7: 28651 accepted, 0
    rejected, 171907 RHS calls; validation.csv: photon integral 1.2128563927511686; grid_timings.csv:7:
    the 9-point detuning grid, 329395 accepted steps, 1976397 RHS calls).  The records predate the
    reference's 0.2.4 X rotational model, which moves the integral by 8.6e-5 relative and the grid
    by one step; the single solve's step and RHS counts are exact."""
    d = golden("plan_r2_38")
    k, kg = d["kat"], d["kat_grid"]
    p = oracle.OraclePlan(d["payload"])
    o = p.options(t0=0.0, t1=d["t_span"][1], abstol=k["abstol"], reltol=k["reltol"], dt=k["dt"], saveat=None,
                  save_start=True, maxiters=100000, solver=k["solver"], output="photon_integral", output_indices=None,
                  output_when="final", integral_weights=[tuple(w) for w in k["weights"]], stop_event=None)
    _, v, st = p.solve_single(o, d["rho0_packed"])
    assert (st["accepted_steps"], st["rejected_steps"], st["rhs_calls"]) == (k["accepted_steps"], 0, k["rhs_calls"])
    assert abs(float(np.asarray(v).reshape(-1)[0]) / k["photon_integral"] - 1.0) < 1e-4
    _, _, gst = p.solve_batch(o, d["rho0_packed"], [p.slot_names.index("detuning")],
                              kg["detuning"].reshape(-1, 1).astype(complex))
    assert abs(int(gst["accepted_steps"].sum()) - kg["accepted_steps"]) <= 2
    assert int(gst["rejected_steps"].sum()) == 0
    assert abs(int(gst["rhs_calls"].sum()) - kg["rhs_calls"]) <= 12


@pytest.mark.parametrize("solver", ["tsit5", "dopri5"])
def test_replay_of_an_event_ended_solve(golden, solver):
    """The frozen-step replay (the gradient tests' finite differences) given the steps of an
    event-free solve up to the crossing and `event_hit` reproduces the solve that the stop event
    ends: the same crossing by bisection, the same final integral and populations."""
    d = golden("plan_q1_16_tend")
    op = oracle.OraclePlan(d["payload"])
    g = d["gamma"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [names.index(s) for s in ("rabi", "detuning", "theta", "t_end")]
    w = [(i, 1.0) for i in d["excited_indices"]]
    p = np.array([[1.3 * g, 0.7 * g, 0.4, 123.4 / g]], dtype=complex)
    common = dict(t0=0.0, t1=200 / g, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, maxiters=100000, solver=solver,
                  output_indices=None)
    tt, _, _ = op.solve_single(op.options(saveat=None, save_start=True, output="populations", output_when="saveat",
                                          integral_weights=None, stop_event=None, **common),
                               d["rho0_packed"], slots, p[0], capacity=100000)
    tt = np.asarray(tt)
    steps = np.stack([tt[:-1], np.diff(tt)], axis=1)
    events = [{"kind": "runtime_expression",
               "expression": {"instructions": [{"op": 4}, {"op": 2, "index": names.index("t_end")}, {"op": 6}],
                              "scalar_only": True, "output_is_tuple": False}},
              {"kind": "population", "indices": list(d["excited_indices"]), "threshold": 0.004}]
    for ev in events:
        for integral in (True, False):
            o = op.options(saveat=None if integral else np.array([200 / g]), save_start=integral,
                           output="excited_population" if integral else "populations", output_when="final",
                           integral_weights=w if integral else None, stop_event=ev, **common)
            vals, _, st = op.solve_batch(o, d["rho0_packed"].reshape(1, -1), slots, p)
            assert st["event_triggered"][0]
            k = int(np.searchsorted(tt, float(st["event_time"][0]), side="left"))
            r = op.solve_replay(o, d["rho0_packed"], slots, p, [steps[:k]], event_hit=[1])
            ref = np.asarray(vals).reshape(-1)
            np.testing.assert_allclose(np.asarray(r).reshape(-1), ref, rtol=1e-13, atol=1e-15 * np.max(np.abs(ref)))
