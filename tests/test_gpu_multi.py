"""GPU parity of the heterogeneous batch (obe_solve_multi_device): batches on plans of 16, 39 and
76 states in one call, with ragged end times from a scanned ``t_end`` feeding a ``Time() - t_end``
stop event.

Each job runs the same kernel, on the same per-trajectory arithmetic, as the single-plan call, so
results and statistics must be bit-identical to solving each batch on its own.  Against the CPU
oracle: event times to 1e-12 relative; smooth drives (16 and 39 states) to 1e-9 relative on the
excited-population integral; the 76-state square-wave drive is discontinuous, so it agrees to the
solver tolerance (5e-6 relative on the integral, as on the single-plan path).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu


def _event(d):
    names = d["payload"]["parameter_graph"]["slot_names"]
    return {"kind": "runtime_expression",
            "expression": {"instructions": [{"op": 4}, {"op": 2, "index": names.index("t_end")}, {"op": 6}],
                           "scalar_only": True, "output_is_tuple": False}}


def _job(golden, name, count, seed, t_end_range):
    """One job of the heterogeneous batch: seeded parameters as in the 16-state scan (peak Rabi
    log-uniform in [0.1, 10] Γ, detuning U[-5, 5] Γ, polarisation angle U[0, π]) or, for the 76-state
    system, per-laser Rabi U[0.5, 3] Γ and detuning N(0, 0.5 Γ); end times uniform in t_end_range / Γ."""
    d = golden(name)
    g = d["gamma"]
    rng = np.random.default_rng(seed)
    names = d["payload"]["parameter_graph"]["slot_names"]
    if name == "plan_rc_76":
        slot_names = ["Ω0", "Ω1", "δ0", "δ1", "t_end"]
        cols = [rng.uniform(0.5, 3.0, count) * g, rng.uniform(0.5, 3.0, count) * g,
                rng.normal(0.0, 0.5, count) * g, rng.normal(0.0, 0.5, count) * g]
    else:
        slot_names = ["rabi", "detuning", "theta", "t_end"]
        cols = [g * 10 ** rng.uniform(-1.0, 1.0, count), rng.uniform(-5.0, 5.0, count) * g,
                rng.uniform(0.0, np.pi, count)]
    t_end = rng.uniform(*t_end_range, count) / g
    params = np.stack(cols + [t_end], axis=1).astype(np.complex128)
    w = [(i, 1.0) for i in d["excited_indices"]]
    job = dict(plan=api.prepare_lindblad_problem_py(d["payload"]),
               packed_rho0_batch=np.repeat(d["rho0_packed"].reshape(1, -1), count, axis=0),
               t0=0.0, t1=1.01 * t_end_range[1] / g, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, solver="tsit5",
               output="excited_population", integral_weights=w,
               parameter_slot_indices=[names.index(s) for s in slot_names], parameter_batch=params,
               stop_event=_event(d))
    return d, job, t_end


@pytest.fixture(scope="module")
def jobs(golden):
    return [_job(golden, "plan_q1_16_tend", 96, 1, (5.0, 30.0)),
            _job(golden, "plan_r0_39", 40, 2, (5.0, 30.0)),
            _job(golden, "plan_rc_76", 12, 3, (5.0, 12.0))]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_batch_is_bit_identical_to_single_plan_calls(jobs, precision):
    out = api.solve_lindblad_multi_batch_ode_py([j for _, j, _ in jobs], precision=precision)
    assert len(out) == len(jobs)
    for (d, job, t_end), (times, values, width, tc, st) in zip(jobs, out):
        rt, rv, rw, rtc, rst = api.solve_lindblad_batch_ode_py(**job, precision=precision)
        assert (width, tc) == (rw, rtc) == (1, 1)
        np.testing.assert_array_equal(values, rv)
        np.testing.assert_array_equal(times, rt)
        for key in ("accepted_steps", "rejected_steps", "rhs_calls", "event_count"):
            assert st[key] == rst[key]
        assert all(st["event_triggered_by_trajectory"])
        np.testing.assert_allclose(np.asarray(st["event_times"]), t_end, rtol=1e-12)


def test_multi_batch_matches_oracle(jobs):
    out = api.solve_lindblad_multi_batch_ode_py([j for _, j, _ in jobs])
    for (d, job, t_end), (_, values, _, _, st) in zip(jobs, out):
        op = oracle.OraclePlan(d["payload"])
        take = slice(0, 6)
        o = op.options(t0=job["t0"], t1=job["t1"], abstol=job["abstol"], reltol=job["reltol"], dt=job["dt"],
                       saveat=None, save_start=True, maxiters=100000, solver="tsit5", output="excited_population",
                       output_indices=None, output_when="final", integral_weights=job["integral_weights"],
                       stop_event=job["stop_event"])
        ref, rt, rst = op.solve_batch(o, job["packed_rho0_batch"][take], job["parameter_slot_indices"],
                                      job["parameter_batch"][take])
        rtol = 5e-6 if d["payload"]["n_states"] == 76 else 1e-9
        np.testing.assert_allclose(np.asarray(values)[take], ref.reshape(-1), rtol=rtol, atol=0.0)
        np.testing.assert_allclose(np.asarray(st["event_times"])[take], t_end[take], rtol=1e-12)


def test_multi_batch_mixed_precision_error(jobs):
    """The mixed form stays within the 1e-6 population bar of the FP64 form, job by job: the
    integral's difference over the integration time is a time-averaged population difference
    (the integrals themselves are down to 1e-19 s, so a relative bar on them says nothing)."""
    a = api.solve_lindblad_multi_batch_ode_py([j for _, j, _ in jobs])
    b = api.solve_lindblad_multi_batch_ode_py([j for _, j, _ in jobs], precision="mixed")
    for (_, _, t_end), (_, va, _, _, _), (_, vb, _, _, _) in zip(jobs, a, b):
        va, vb = np.asarray(va), np.asarray(vb)
        assert np.max(np.abs(vb - va) / t_end) < 1e-6
        assert not np.array_equal(va, vb)  # the two forms really are different arithmetic


def test_multi_batch_errors(jobs):
    (_, j16, _), (_, j39, _), _ = jobs
    with pytest.raises(ValueError, match=r"^job 1: plan already used by job 0 \(one job per plan\)$"):
        api.solve_lindblad_multi_batch_ode_py([j16, dict(j16)])
    bad = dict(j39, maxiters=3)
    with pytest.raises(ValueError, match=r"^job 1: trajectory 0: "):
        api.solve_lindblad_multi_batch_ode_py([j16, bad])
    # an empty job is allowed and returns the single-plan call's empty result
    empty = dict(j16, packed_rho0_batch=np.zeros((0, 256)), parameter_batch=np.zeros((0, 4), complex))
    out = api.solve_lindblad_multi_batch_ode_py([empty, j39])
    assert out[0][3] == 0 and out[1][2] == 1


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_multi_graph_replays_the_batch(jobs, precision):
    """obe_multi_graph: the batch recorded once as a CUDA graph gives the immediate call's values
    and statistics bit for bit, and a second launch after the inputs changed in place gives the
    immediate call's results for the new inputs."""
    torch = pytest.importorskip("torch")
    from centrex_tlf_gb300.native import MultiGraph, multi_solve_device

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    built = []
    for _, job, _ in jobs:
        plan = job["plan"].native
        opts = plan.options(t0=job["t0"], t1=job["t1"], abstol=job["abstol"], reltol=job["reltol"], dt=job["dt"],
                            saveat=None, save_start=True, maxiters=100000, solver="tsit5", output="excited_population",
                            output_indices=None, output_when="final", integral_weights=job["integral_weights"],
                            stop_event=job["stop_event"], precision=precision)
        b = job["packed_rho0_batch"].shape[0]
        built.append(dict(plan=plan, opts=opts, b=b, slots=job["parameter_slot_indices"],
                          rho=torch.from_numpy(job["packed_rho0_batch"]).to(dev),
                          par=torch.from_numpy(np.ascontiguousarray(job["parameter_batch"]).view(np.float64).reshape(-1)).to(dev),
                          val=torch.zeros(b, dtype=torch.float64, device=dev), st=torch.zeros(b * 6, dtype=torch.int64, device=dev),
                          ref=torch.zeros(b, dtype=torch.float64, device=dev), rst=torch.zeros(b * 6, dtype=torch.int64, device=dev)))

    def spec(out, stats):
        return [(x["plan"], x["opts"], x["b"], x["rho"].data_ptr(), x["slots"], x["par"].data_ptr(), 1, x[out].data_ptr(),
                 x[stats].data_ptr()) for x in built]

    graph = MultiGraph(spec("val", "st"))
    try:
        for rep in range(2):
            if rep == 1:
                for x in built:
                    x["par"].view(x["b"], -1, 2)[:, 0, 0] *= 1.3  # the first scanned slot: a Rabi rate
            assert graph.launch(stream) == len(built)
            multi_solve_device(spec("ref", "rst"), stream)
            torch.cuda.synchronize()
            for x in built:
                assert torch.equal(x["val"], x["ref"])
                assert torch.equal(x["st"], x["rst"])
                assert not bool((x["st"].view(-1, 6)[:, 3] >> 32).any())
    finally:
        graph.close()


def test_multi_graph_survives_other_calls_and_refuses_a_relaid_plan(jobs):
    """The graph owns its stage buffers: a larger solve on the same 76-state plan between two
    launches (which grows the plan's own buffers) leaves the graph's results unchanged.  A plan
    laid out again (a new launch shape, hence a new device image) makes the graph refuse to
    launch until it is recorded again."""
    torch = pytest.importorskip("torch")
    from centrex_tlf_gb300.native import MultiGraph

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    built = []
    for _, job, _ in jobs:
        plan = job["plan"].native
        opts = plan.options(t0=job["t0"], t1=job["t1"], abstol=job["abstol"], reltol=job["reltol"], dt=job["dt"],
                            saveat=None, save_start=True, maxiters=100000, solver="tsit5", output="excited_population",
                            output_indices=None, output_when="final", integral_weights=job["integral_weights"],
                            stop_event=job["stop_event"], precision="mixed")
        b = job["packed_rho0_batch"].shape[0]
        built.append(dict(plan=plan, opts=opts, b=b, slots=job["parameter_slot_indices"], job=job,
                          rho=torch.from_numpy(job["packed_rho0_batch"]).to(dev),
                          par=torch.from_numpy(np.ascontiguousarray(job["parameter_batch"]).view(np.float64).reshape(-1)).to(dev),
                          val=torch.zeros(b, dtype=torch.float64, device=dev), st=torch.zeros(b * 6, dtype=torch.int64, device=dev)))
    spec = [(x["plan"], x["opts"], x["b"], x["rho"].data_ptr(), x["slots"], x["par"].data_ptr(), 1, x["val"].data_ptr(),
             x["st"].data_ptr()) for x in built]
    graph = MultiGraph(spec)
    try:
        graph.launch(stream)
        torch.cuda.synchronize()
        first = [x["val"].clone() for x in built]
        # a larger batch on the 76-state plan through the ordinary call
        big = built[-1]
        reps = 160 // big["b"] + 1
        job = dict(big["job"], packed_rho0_batch=np.tile(big["job"]["packed_rho0_batch"], (reps, 1)),
                   parameter_batch=np.tile(big["job"]["parameter_batch"], (reps, 1)))
        api.solve_lindblad_batch_ode_py(**job, precision="mixed")
        graph.launch(stream)
        torch.cuda.synchronize()
        for x, v in zip(built, first):
            assert torch.equal(x["val"], v)
        # a new launch shape for the 16-state plan: its device image is rebuilt
        p16 = built[0]["plan"]
        old = p16.shape()
        p16.set_shape(64, 0)
        with pytest.raises(ValueError, match="laid out again"):
            graph.launch(stream)
        p16.set_shape(*old)
        with pytest.raises(ValueError, match="laid out again"):
            graph.launch(stream)
    finally:
        graph.close()
    graph = MultiGraph(spec)  # recorded again: launches
    try:
        assert graph.launch(stream) == len(built)
        torch.cuda.synchronize()
        for x, v in zip(built, first):
            assert torch.equal(x["val"], v)
    finally:
        graph.close()
