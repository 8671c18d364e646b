"""GPU parity on the reference's heavy known answer: the 38-state R(2) benchmark system
(128 threads per trajectory), one Dopri5 solve of 28,651 steps and the 9-point detuning grid.

Against the oracle: the same step and RHS counts to 0.1 % and the photon integral to 1e-7
relative -- a long solve whose rounding-level differences (fused multiply-adds, summation order)
can move a step decision; against the reference's own records: the counts to 0.1 %.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def r2(golden):
    d = golden("plan_r2_38")
    k = d["kat"]
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=0.0, t1=d["t_span"][1], abstol=k["abstol"], reltol=k["reltol"], dt=k["dt"], saveat=None,
                   save_start=True, maxiters=100000, solver=k["solver"], output="photon_integral", output_indices=None,
                   output_when="final", integral_weights=[tuple(w) for w in k["weights"]], stop_event=None)
    return d, api.prepare_lindblad_problem_py(d["payload"]), op, o


def _close(a, b, rel):
    return abs(a - b) <= rel * b


def test_r2_38_single_solve(r2):
    d, plan, op, o = r2
    k = d["kat"]
    _, v, w, st = api.solve_lindblad_ode_py(plan, d["rho0_packed"], 0.0, d["t_span"][1], k["abstol"], k["reltol"], k["dt"],
                                            None, True, 100000, "expanded_sparse", "dopri5", "photon_integral", None,
                                            "final", [tuple(x) for x in k["weights"]], None)
    _, rv, rst = op.solve_single(o, d["rho0_packed"])
    val, ref = float(np.asarray(v).reshape(-1)[0]), float(np.asarray(rv).reshape(-1)[0])
    assert abs(val - ref) <= 1e-7 * ref
    for key in ("accepted_steps", "rhs_calls"):
        assert _close(st[key], rst[key], 1e-3) and _close(st[key], k[key], 1e-3)
    assert abs(val / k["photon_integral"] - 1.0) < 1e-4


def test_r2_38_detuning_grid(r2):
    d, plan, op, o = r2
    k, kg = d["kat"], d["kat_grid"]
    slot = d["payload"]["parameter_graph"]["slot_names"].index("detuning")
    axis = kg["detuning"].astype(complex)
    _, gv, _, _, gst = api.solve_lindblad_grid_ode_py(
        plan, d["rho0_packed"], 0.0, d["t_span"][1], k["abstol"], k["reltol"], k["dt"], [slot], axis, [axis.size],
        solver="dopri5", output="photon_integral", integral_weights=[tuple(x) for x in k["weights"]])
    ref, _, rst = op.solve_batch(o, d["rho0_packed"], [slot], axis.reshape(-1, 1))
    np.testing.assert_allclose(np.asarray(gv).reshape(-1), ref.reshape(-1), rtol=1e-7)
    assert _close(gst["accepted_steps"], int(rst["accepted_steps"].sum()), 1e-3)
    assert _close(gst["accepted_steps"], kg["accepted_steps"], 1e-3)
    assert _close(gst["rhs_calls"], kg["rhs_calls"], 1e-3)
