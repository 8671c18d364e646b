"""The multi-device batch driver on the GPU this run has: the batch cut into slices that two host
threads solve concurrently, each through its own plan (device 0 twice stands in for two GPUs),
gathers to exactly the one-call result, first error included."""

from __future__ import annotations

import numpy as np
import pytest

from centrex_tlf_gb300 import centrex_tlf_rust as api
from centrex_tlf_gb300.multigpu import solve_batch_across_devices

pytestmark = pytest.mark.gpu


def test_batch_across_devices_equals_one_call(golden):
    d = golden("plan_q1_16")
    g, (t0, t1) = d["gamma"], d["t_span"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [names.index(s) for s in ("rabi", "detuning", "theta")]
    rng = np.random.default_rng(3)
    b = 37
    params = np.stack([g * 10 ** rng.uniform(-1, 1, b), rng.uniform(-5, 5, b) * g, rng.uniform(0, np.pi, b)],
                      axis=1).astype(np.complex128)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0)
    kw = dict(solver="tsit5", output="populations", parameter_slot_indices=slots)
    plan = api.prepare_lindblad_problem_py(d["payload"])
    one = api.solve_lindblad_batch_ode_py(plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / g, parameter_batch=params, **kw)
    costs = np.linspace(1.0, 3.0, b)
    for devices, c in (([0, 0], None), ([0, 0, 0], costs)):
        many = solve_batch_across_devices(d["payload"], rho0, t0, t1, 1e-11, 1e-8, 1e-3 / g, devices=devices,
                                          costs=c, parameter_batch=params, **kw)
        np.testing.assert_array_equal(many[0], one[0])
        np.testing.assert_array_equal(many[1], one[1])
        assert many[2:4] == one[2:4]
        assert many[4] == one[4]
    # the first failing trajectory keeps its index in the whole batch
    with pytest.raises(ValueError, match=r"^trajectory 0: Stopped at x="):
        api.solve_lindblad_batch_ode_py(plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / g, parameter_batch=params, maxiters=3, **kw)
    with pytest.raises(ValueError, match=r"^trajectory 0: Stopped at x="):
        solve_batch_across_devices(d["payload"], rho0, t0, t1, 1e-11, 1e-8, 1e-3 / g, devices=[0, 0],
                                   parameter_batch=params, maxiters=3, **kw)
