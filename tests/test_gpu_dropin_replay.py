"""The drop-in, call by call: every native call that the reference's own Python surface makes
(recorded in ``tests/golden/ffi_calls.json`` by running the reference's ``solve_lindblad``
(solve.py:419), ``parameter_scan`` / ``solve_lindblad_batch`` (batch.py:235) and ``grid_scan``
(batch.py:440) against a recording stand-in for ``centrex_tlf.centrex_tlf_rust``) is replayed
with exactly those positional arguments through this package's ``centrex_tlf_rust`` module on the
GPU, and each result is compared with the oracle.

The oracle's options follow the reference's option mapping (python_api.rs:589-617, 723-746),
restated here independently of the shim: ``output_when="final"`` with a non-integral output
saves at ``[t1]`` only, without the start point; a final integral keeps saveat and save_start.

Tolerances: populations and selected elements 1e-9 absolute, integrals 1e-8 relative (FP64
solves whose controllers see the same error estimates up to rounding).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu

INTEGRALS = ("weighted_integral", "photon_integral", "excited_population")


@pytest.fixture(scope="module")
def replay(golden):
    d = golden("plan_q1_16")
    calls = golden("ffi_calls")
    assert calls["slot_names"] == d["payload"]["parameter_graph"]["slot_names"]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    return d, plan, oracle.OraclePlan(d["payload"]), calls["calls"]


def _oracle_opts(op, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output, output_indices,
                 output_when, integral_weights, stop_event):
    final_integral = output_when == "final" and output in INTEGRALS
    if output_when == "final" and not final_integral:
        saveat, save_start = np.array([t1]), False
    return op.options(t0=t0, t1=t1, abstol=abstol, reltol=reltol, dt=dt, saveat=saveat, save_start=save_start,
                      maxiters=maxiters, solver=solver, output=output, output_indices=output_indices,
                      output_when=output_when, integral_weights=integral_weights, stop_event=stop_event)


def _compare(output, got, ref):
    got = np.asarray(got).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    assert got.shape == ref.shape
    assert np.all(np.isfinite(got))
    if output in INTEGRALS:
        np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-20)
    else:
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9)


def _calls(replay, fn):
    return [c["args"] for c in replay[3] if c["fn"] == fn]


def test_every_recorded_call_is_replayed(replay):
    kinds = sorted({c["fn"] for c in replay[3]})
    assert kinds == ["solve_lindblad_batch_ode_py", "solve_lindblad_grid_ode_py", "solve_lindblad_ode_py"]
    assert len(replay[3]) == 6


def test_single_solves_match_oracle(replay):
    d, plan, op, _ = replay
    calls = _calls(replay, "solve_lindblad_ode_py")
    assert len(calls) == 3
    for args in calls:
        (rho0, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, mode, solver, output, output_indices,
         output_when, integral_weights, stop_event, _split) = args
        times, values, width, stats = api.solve_lindblad_ode_py(plan, *args)
        assert stats["solver"] == solver and stats["accepted_steps"] > 0
        o = _oracle_opts(op, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output,
                         output_indices, output_when, integral_weights, stop_event)
        rt, rv, rst = op.solve_single(o, rho0)
        assert width == rv.shape[1]
        np.testing.assert_allclose(times, rt, rtol=0, atol=1e-18)
        _compare(output, values, rv)
        assert abs(stats["accepted_steps"] - rst["accepted_steps"]) <= 0.02 * rst["accepted_steps"] + 2


def test_batch_solves_match_oracle(replay):
    d, plan, op, _ = replay
    calls = _calls(replay, "solve_lindblad_batch_ode_py")
    assert len(calls) == 2
    for args in calls:
        (rho0, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, mode, solver, output, output_indices,
         output_when, integral_weights, slots, pbatch, _par, _threads, stop_event, _split) = args
        times, values, width, tc, stats = api.solve_lindblad_batch_ode_py(plan, *args)
        o = _oracle_opts(op, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output,
                         output_indices, output_when, integral_weights, stop_event)
        ref, rtimes, rst = op.solve_batch(o, rho0, slots, pbatch, time_count=tc)
        assert len(stats["event_triggered_by_trajectory"]) == rho0.shape[0]
        np.testing.assert_allclose(times, rtimes, rtol=0, atol=1e-18)
        _compare(output, values, ref)
        assert abs(stats["accepted_steps"] - int(rst["accepted_steps"].sum())) <= 0.02 * int(rst["accepted_steps"].sum()) + 2


def test_grid_solve_matches_oracle(replay):
    """The grid's trajectory order is row-major with the last axis fastest
    (ode_batch.rs:369-391); the oracle gets the same points as an explicit batch."""
    d, plan, op, _ = replay
    (args,) = _calls(replay, "solve_lindblad_grid_ode_py")
    (rho0, t0, t1, abstol, reltol, dt, slots, axes, lengths, saveat, save_start, maxiters, mode, solver, output,
     output_indices, output_when, integral_weights, _par, _threads, stop_event, _split) = args
    times, values, width, tc, stats = api.solve_lindblad_grid_ode_py(plan, *args)
    axes = np.asarray(axes, dtype=np.complex128)
    split = np.split(axes, np.cumsum(lengths)[:-1])
    points = np.array([[a, b] for a in split[0] for b in split[1]], dtype=np.complex128)
    assert len(stats["event_triggered_by_trajectory"]) == points.shape[0]
    o = _oracle_opts(op, t0, t1, abstol, reltol, dt, saveat, save_start, maxiters, solver, output, output_indices,
                     output_when, integral_weights, stop_event)
    ref, _, _ = op.solve_batch(o, rho0, slots, points, time_count=tc)
    _compare(output, values, ref)
