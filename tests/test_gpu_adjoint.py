"""GPU gradients (centrex_tlf_gb300.autograd over obe_grad_forward / obe_grad_backward) against
central finite differences of the CPU oracle replaying the same frozen step sequence, for the
16-, 39- and 76-state systems, full and checkpointed tapes.

The adjoint differentiates the discrete solve with its accepted steps frozen, so the check is
the oracle's replay of exactly those steps at p +- eps (eps = 1e-6 |p|): agreement to 1e-5
relative, plus a floor for the differences' rounding -- the loss carries ~1e-14 relative rounding
from some thousand steps, i.e. ~1e-8 of its natural scale |J| / |p| once divided by eps (this
matters for derivatives that are nearly zero, such as the final populations' dependence on the
pulse centre when the pulse ends long before t1).  The loss is linear in the initial state, so
its differences there use a unit step and are exact up to rounding.  The forward values equal
the plain FP64 solve's; the oracle's replay at p reproduces them to 1e-10.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from centrex_tlf_gb300.autograd import solve_batch_with_grad  # noqa: E402
from centrex_tlf_gb300.native import NativePlan  # noqa: E402

W = [(13, 1.0), (14, 1.0), (15, 1.0)]


@pytest.fixture(scope="module")
def q1(golden):
    d = golden("plan_q1_16")
    return d, NativePlan(d["payload"]), oracle.OraclePlan(d["payload"])


def _params(d):
    g = d["gamma"]
    # rabi, detuning, theta, t_center for four points of the benchmark's distribution
    return np.array([[1.0 * g, 0.0, 0.3, 100.0 / g], [3.0 * g, -2.0 * g, 1.1, 95.0 / g],
                     [0.4 * g, 1.5 * g, 2.5, 104.0 / g], [6.0 * g, 4.0 * g, 0.8, 100.0 / g]])


def _slots(d, names=("rabi", "detuning", "theta", "t_center")):
    return [d["payload"]["parameter_graph"]["slot_names"].index(s) for s in names]


def _oracle_opts(op, d, solver, output):
    t0, t1 = d["t_span"]
    g = d["gamma"]
    if output == "populations":
        return op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([t1]), save_start=False,
                          maxiters=100000, solver=solver, output="populations", output_indices=None, output_when="final",
                          integral_weights=None, stop_event=None)
    return op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None, save_start=True, maxiters=100000,
                      solver=solver, output="excited_population", output_indices=None, output_when="final",
                      integral_weights=W, stop_event=None)


@pytest.mark.parametrize("solver,output", [("tsit5", "excited_population"), ("dopri5", "excited_population"),
                                           ("tsit5", "populations")])
def test_parameter_gradients_match_frozen_step_finite_differences(q1, solver, output):
    d, plan, op = q1
    g = d["gamma"]
    slots = _slots(d)
    p0 = _params(d)
    b = p0.shape[0]
    params = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    out, tape = solve_batch_with_grad(plan, d["rho0_packed"], d["t_span"], params, slots, solver=solver,
                                      dt=1e-3 / g, output=output, integral_weights=W if output != "populations" else None,
                                      return_tape=True)
    rng = np.random.default_rng(3)
    wout = rng.normal(size=(b, 16)) if output == "populations" else np.ones((b, 1))
    loss = (out.reshape(b, -1) * torch.tensor(wout, device="cuda")).sum()
    loss.backward()
    grad = params.grad.cpu().numpy()
    steps = tape.steps()
    # the forward values are the plain FP64 solve's
    _, ref_vals, _, _, _ = api.solve_lindblad_batch_ode_py(
        api.prepare_lindblad_problem_py(d["payload"]), np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0),
        d["t_span"][0], d["t_span"][1], 1e-11, 1e-8, 1e-3 / g, solver=solver,
        output=output, integral_weights=W if output != "populations" else None, parameter_slot_indices=slots,
        parameter_batch=p0.astype(complex))
    np.testing.assert_allclose(out.detach().cpu().numpy().reshape(-1), np.asarray(ref_vals).reshape(-1), rtol=1e-12, atol=1e-20)
    o = _oracle_opts(op, d, solver, output)
    rho0 = d["rho0_packed"]

    def replay(p):
        v = op.solve_replay(o, rho0, slots, p.astype(complex), steps)
        return (np.asarray(v).reshape(b, -1) * wout).sum(axis=1)

    base = replay(p0)
    np.testing.assert_allclose(base, (out.detach().cpu().numpy().reshape(b, -1) * wout).sum(axis=1), rtol=1e-10, atol=1e-22)
    for k in range(p0.shape[1]):
        eps = 1e-6 * np.abs(p0[:, k])
        eps[eps == 0] = 1e-6 * (g if k == 1 else 1.0)
        pp, pm = p0.copy(), p0.copy()
        pp[:, k] += eps
        pm[:, k] -= eps
        fd = (replay(pp) - replay(pm)) / (2 * eps)
        natural = np.abs(base) / np.maximum(np.abs(p0[:, k]), 1e-300)
        tol = 1e-5 * np.abs(fd) + 1e-8 * natural
        assert np.all(np.abs(grad[:, k] - fd) <= tol), (k, grad[:, k], fd, tol)


def _fd_check(d, plan, op, p0, slots, solver="tsit5", t_span=None, weights=None, checkpoint_every=0):
    """Gradients of the excited-population integral against central differences of the oracle's
    replay of the frozen steps (the bar of the test above)."""
    g = d["gamma"]
    t_span = d["t_span"] if t_span is None else t_span
    w = weights if weights is not None else [(i, 1.0) for i in d["excited_indices"]]
    b = p0.shape[0]
    params = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    out, tape = solve_batch_with_grad(plan, d["rho0_packed"], t_span, params, slots, solver=solver, dt=1e-3 / g,
                                      integral_weights=w, return_tape=True, checkpoint_every=checkpoint_every)
    assert tape.checkpoint_every == checkpoint_every
    out.sum().backward()
    grad = params.grad.cpu().numpy()
    steps = tape.steps()
    o = op.options(t0=t_span[0], t1=t_span[1], abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None, save_start=True,
                   maxiters=100000, solver=solver, output="excited_population", output_indices=None,
                   output_when="final", integral_weights=w, stop_event=None)

    def replay(p):
        return np.asarray(op.solve_replay(o, d["rho0_packed"], slots, p.astype(complex), steps)).reshape(b)

    base = replay(p0)
    np.testing.assert_allclose(base, out.detach().cpu().numpy().reshape(-1), rtol=1e-10, atol=1e-22)
    for k in range(p0.shape[1]):
        eps = 1e-6 * np.abs(p0[:, k])
        eps[eps == 0] = 1e-6 * g
        pp, pm = p0.copy(), p0.copy()
        pp[:, k] += eps
        pm[:, k] -= eps
        fd = (replay(pp) - replay(pm)) / (2 * eps)
        tol = 1e-5 * np.abs(fd) + 1e-8 * np.abs(base) / np.maximum(np.abs(p0[:, k]), 1e-300)
        assert np.all(np.abs(grad[:, k] - fd) <= tol), (k, grad[:, k], fd, tol)


@pytest.mark.parametrize("tpt", [64, 128])
def test_gradients_at_wider_launch_shapes(q1, tpt):
    """The 16-state plan laid out for 64 or 128 threads per trajectory (what the autotuner picks
    for small batches): the adjoint runs at that width too and matches the finite differences."""
    d, plan, op = q1
    plan.set_shape(tpt, 0)
    try:
        _fd_check(d, plan, op, _params(d)[:3], _slots(d))
    finally:
        plan.set_shape(0, 0)


def test_gradients_of_the_39_state_system(golden):
    """X J=0-2 + B (39 states, 128 threads per trajectory): gradients with respect to the peak
    Rabi rate, detuning, polarisation angle and pulse centre over [0, 150/Γ]."""
    d = golden("plan_r0_39")
    g = d["gamma"]
    plan = NativePlan(d["payload"])
    assert plan.shape()[0] == 128
    op = oracle.OraclePlan(d["payload"])
    p0 = np.array([[1.5 * g, 0.5 * g, 0.4, 70.0 / g], [4.0 * g, -1.0 * g, 1.2, 75.0 / g]])
    _fd_check(d, plan, op, p0, _slots(d), t_span=(0.0, 150.0 / g))


@pytest.mark.parametrize("ck", [7, 512])
def test_checkpointed_tape_matches_the_full_tape(q1, ck):
    """Checkpoints every C accepted steps, segments replayed in the reverse sweep: the same
    gradients as the full tape up to the replay's rounding, for parameters and the initial state,
    and the finite differences of the frozen steps."""
    d, plan, op = q1
    g = d["gamma"]
    slots = _slots(d)
    p0 = _params(d)[:3]
    res = {}
    for c in (0, ck):
        params = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
        rho0 = torch.tensor(np.repeat(d["rho0_packed"].reshape(1, -1), 3, axis=0), dtype=torch.float64, device="cuda",
                            requires_grad=True)
        out, tape = solve_batch_with_grad(plan, rho0, d["t_span"], params, slots, dt=1e-3 / g, integral_weights=W,
                                          return_tape=True, checkpoint_every=c)
        out.sum().backward()
        res[c] = (out.detach().cpu().numpy(), params.grad.cpu().numpy(), rho0.grad.cpu().numpy(), tape.tape.numel())
    np.testing.assert_array_equal(res[ck][0], res[0][0])  # the same forward solve
    np.testing.assert_allclose(res[ck][1], res[0][1], rtol=1e-9, atol=0.0)
    np.testing.assert_allclose(res[ck][2], res[0][2], rtol=1e-9, atol=1e-12 * np.max(np.abs(res[0][2])))
    assert res[ck][3] < res[0][3] / 5  # 2 + N / C doubles per step instead of 2 + 7 N
    _fd_check(d, plan, op, p0, slots, checkpoint_every=ck)


@pytest.mark.parametrize("ck", [0, 16])
def test_gradients_of_the_76_state_system(golden, ck):
    """The 76-state system (256 threads per trajectory; the adjoint's mu, ybar and class sums in
    device memory), square-wave polarisations: gradients of the excited-population integral over
    [0, 6/Γ] with respect to both lasers' Rabi rates and detunings, full and checkpointed tape."""
    d = golden("plan_rc_76")
    g = d["gamma"]
    plan = NativePlan(d["payload"])
    assert plan.shape()[0] == 256
    op = oracle.OraclePlan(d["payload"])
    p0 = np.array([[1.2 * g, 2.0 * g, 0.3 * g, -0.2 * g], [2.5 * g, 0.8 * g, -0.4 * g, 0.6 * g]])
    _fd_check(d, plan, op, p0, _slots(d, ("Ω0", "Ω1", "δ0", "δ1")), t_span=(0.0, 6.0 / g), checkpoint_every=ck)


def test_initial_state_gradient_matches_finite_differences(q1):
    d, plan, op = q1
    g = d["gamma"]
    slots = _slots(d)
    p0 = _params(d)[:2]
    rho0 = torch.tensor(np.repeat(d["rho0_packed"].reshape(1, -1), 2, axis=0), dtype=torch.float64, device="cuda",
                        requires_grad=True)
    params = torch.tensor(p0, dtype=torch.float64, device="cuda")
    out, tape = solve_batch_with_grad(plan, rho0, d["t_span"], params, slots, dt=1e-3 / g, output="excited_population",
                                      integral_weights=W, return_tape=True)
    out.sum().backward()
    gr = rho0.grad.cpu().numpy()
    steps = tape.steps()
    o = _oracle_opts(op, d, "tsit5", "excited_population")
    base = np.repeat(d["rho0_packed"].reshape(1, -1), 2, axis=0)
    j0 = op.solve_replay(o, base, slots, p0.astype(complex), steps)
    for idx in (0, 5, 13, 40):  # populations and a coherence component
        ep, em = base.copy(), base.copy()
        ep[:, idx] += 1.0
        em[:, idx] -= 1.0
        fd = (op.solve_replay(o, ep, slots, p0.astype(complex), steps)
              - op.solve_replay(o, em, slots, p0.astype(complex), steps)) / 2.0
        np.testing.assert_allclose(gr[:, idx], fd, rtol=1e-6, atol=1e-12 * np.max(np.abs(j0)))


def test_gradient_errors(golden, q1):
    d, plan, _ = q1
    params = torch.tensor(_params(d)[:1], dtype=torch.float64, device="cuda", requires_grad=True)
    with pytest.raises(NotImplementedError):
        solve_batch_with_grad(plan, d["rho0_packed"], d["t_span"], params, _slots(d), output="selected")
    # a derivative through a helper function's argument is refused, per trajectory
    td = golden("plan_two_level_td")
    tplan = NativePlan(td["payload"])
    names = td["payload"]["parameter_graph"]["slot_names"]
    p = torch.tensor([[0.5]], dtype=torch.float64, device="cuda", requires_grad=True)
    out = solve_batch_with_grad(tplan, td["rho0_packed"], (0.0, 1.0), p, [names.index("modulation_depth")],
                                dt=1e-3, output="populations")
    with pytest.raises(ValueError, match="helper function"):
        out.sum().backward()
    # the helper's outer factor is fine
    p = torch.tensor([[1.0]], dtype=torch.float64, device="cuda", requires_grad=True)
    out = solve_batch_with_grad(tplan, td["rho0_packed"], (0.0, 1.0), p, [names.index("omega0")], dt=1e-3,
                                output="populations")
    out[:, 1].sum().backward()
    assert np.isfinite(p.grad.cpu().numpy()).all() and abs(float(p.grad)) > 0


def _t_end_event(names):
    return {"kind": "runtime_expression",
            "expression": {"instructions": [{"op": 4}, {"op": 2, "index": names.index("t_end")}, {"op": 6}],
                           "scalar_only": True, "output_is_tuple": False}}


def _event_fd_check(d, p0, slots, ev, hits_expected, solver="tsit5", output="excited_population", checkpoint_every=0,
                    t1=None):
    """Gradients of a solve that a stop event ends against central differences of the oracle's
    replay of the frozen steps, whose last step finds the event again at p +- eps (the same bar as
    the event-free checks).  The forward values equal the plain solve's with the same event."""
    g = d["gamma"]
    t1 = 200.0 / g if t1 is None else t1
    plan = NativePlan(d["payload"])
    op = oracle.OraclePlan(d["payload"])
    w = [(i, 1.0) for i in d["excited_indices"]]
    integral = output != "populations"
    b = p0.shape[0]
    params = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    out, tape = solve_batch_with_grad(plan, d["rho0_packed"], (0.0, t1), params, slots, solver=solver, dt=1e-3 / g,
                                      output=output, integral_weights=w if integral else None, return_tape=True,
                                      checkpoint_every=checkpoint_every, stop_event=ev)
    hits = tape.event_hits()
    assert hits.tolist() == hits_expected
    rng = np.random.default_rng(11)
    wout = np.ones((b, 1)) if integral else rng.normal(size=(b, d["payload"]["n_states"]))
    (out.reshape(b, -1) * torch.tensor(wout, device="cuda")).sum().backward()
    grad = params.grad.cpu().numpy()
    _, ref_vals, _, _, _ = api.solve_lindblad_batch_ode_py(
        api.prepare_lindblad_problem_py(d["payload"]), np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0), 0.0, t1,
        1e-11, 1e-8, 1e-3 / g, saveat=None if integral else np.array([t1]), save_start=integral, solver=solver,
        output=output, integral_weights=w if integral else None, parameter_slot_indices=slots,
        parameter_batch=p0.astype(complex), stop_event=ev)
    np.testing.assert_allclose(out.detach().cpu().numpy().reshape(-1), np.asarray(ref_vals).reshape(-1), rtol=1e-12, atol=1e-20)
    o = op.options(t0=0.0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None if integral else np.array([t1]),
                   save_start=integral, maxiters=100000, solver=solver, output=output, output_indices=None,
                   output_when="final", integral_weights=w if integral else None, stop_event=ev)
    steps = tape.steps()

    def replay(p):
        v = op.solve_replay(o, d["rho0_packed"], slots, p.astype(complex), steps, event_hit=hits)
        return (np.asarray(v).reshape(b, -1) * wout).sum(axis=1)

    base = replay(p0)
    np.testing.assert_allclose(base, (out.detach().cpu().numpy().reshape(b, -1) * wout).sum(axis=1), rtol=1e-10, atol=1e-22)
    for k in range(p0.shape[1]):
        eps = 1e-6 * np.abs(p0[:, k])
        eps[eps == 0] = 1e-6 * g
        pp, pm = p0.copy(), p0.copy()
        pp[:, k] += eps
        pm[:, k] -= eps
        fd = (replay(pp) - replay(pm)) / (2 * eps)
        tol = 1e-5 * np.abs(fd) + 1e-8 * np.abs(base) / np.maximum(np.abs(p0[:, k]), 1e-300)
        assert np.all(np.abs(grad[:, k] - fd) <= tol), (k, grad[:, k], fd, tol)
    return grad


@pytest.mark.parametrize("solver,output,ck", [("tsit5", "excited_population", 0), ("dopri5", "excited_population", 0),
                                              ("tsit5", "populations", 0), ("dopri5", "populations", 0),
                                              ("tsit5", "excited_population", 7)])
def test_gradients_through_a_time_event(golden, solver, output, ck):
    """A `Time() - t_end` stop event with t_end a differentiated base slot (the ragged end times of
    the heterogeneous scan): gradients with respect to the Rabi rate, detuning, angle and the end
    time itself (the event time's own derivative); one trajectory's t_end lies past t1."""
    d = golden("plan_q1_16_tend")
    g = d["gamma"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [names.index(s) for s in ("rabi", "detuning", "theta", "t_end")]
    p0 = np.array([[1.0 * g, 0.0, 0.3, 123.4 / g], [3.0 * g, -2.0 * g, 1.1, 60.3 / g], [0.4 * g, 1.5 * g, 2.5, 250.0 / g],
                   [6.0 * g, 4.0 * g, 0.8, 170.7 / g]])
    grad = _event_fd_check(d, p0, slots, _t_end_event(names), [1, 1, 0, 1], solver=solver, output=output,
                           checkpoint_every=ck)
    assert grad[2, 3] == 0.0  # no event, no dependence on t_end
    assert np.all(np.abs(grad[[0, 1, 3], 3]) > 0.0)


@pytest.mark.parametrize("output,ck", [("excited_population", 0), ("populations", 0), ("excited_population", 5)])
def test_gradients_through_a_population_event(golden, output, ck):
    """A threshold on the excited populations ends each trajectory at a state-dependent time: the
    implicit-function term moves ybar at the crossing along the event's population vector."""
    d = golden("plan_q1_16")
    g = d["gamma"]
    slots = _slots(d)
    ev = {"kind": "population", "indices": list(d["excited_indices"]), "threshold": 0.004}
    p0 = np.array([[1.3 * g, 0.7 * g, 0.4, 100.0 / g], [3.0 * g, -2.0 * g, 1.1, 95.0 / g], [0.1 * g, 4.5 * g, 2.5, 104.0 / g]])
    _event_fd_check(d, p0, slots, ev, [1, 1, 0], output=output, checkpoint_every=ck)


def _mixed_fd_check(d, plan, op, p0, slots, t_span, output="excited_population", checkpoint_every=0, stop_event=None,
                    hits_expected=None, rel=1e-5, floor=2e-6):
    """The mixed form (single-precision RHS and reverse-sweep products, double-precision state and
    accumulation) against central differences of the double-precision replay of the mixed
    forward's own frozen steps: 1e-5 relative, with a floor of 2e-6 of the natural scale |J|/|p|.
    The sweep linearises around the mixed forward's states (within ~1e-8 relative of the double
    replay's) rounded to single precision for its products, so a derivative that cancels to ~1e-4
    of its natural scale (the pulse centre's) carries errors of a few 1e-7 of |J|/|p| (measured
    3.4e-7 to 9.6e-7; 0.5e-7 to 6.4e-7 with k_1 refreshed in double every step, which shows the
    forward states' share); the Rabi rate, detuning and angle derivatives agree to ~3e-6
    relative."""
    g = d["gamma"]
    integral = output != "populations"
    w = [(i, 1.0) for i in d["excited_indices"]]
    b = p0.shape[0]
    params = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    out, tape = solve_batch_with_grad(plan, d["rho0_packed"], t_span, params, slots, solver="tsit5", dt=1e-3 / g,
                                      output=output, integral_weights=w if integral else None, return_tape=True,
                                      checkpoint_every=checkpoint_every, stop_event=stop_event, precision="mixed")
    hits = tape.event_hits()
    if hits_expected is not None:
        assert hits.tolist() == hits_expected
    rng = np.random.default_rng(5)
    wout = np.ones((b, 1)) if integral else rng.normal(size=(b, d["payload"]["n_states"]))
    (out.reshape(b, -1) * torch.tensor(wout, device="cuda")).sum().backward()
    grad = params.grad.cpu().numpy()
    # the forward values are the mixed solve's (the same plan, so the same launch shape)
    _, ref_vals, _, _, _ = api.solve_lindblad_batch_ode_py(
        plan, np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0), t_span[0],
        t_span[1], 1e-11, 1e-8, 1e-3 / g, saveat=None if integral else np.array([t_span[1]]), save_start=integral,
        solver="tsit5", output=output, integral_weights=w if integral else None, parameter_slot_indices=slots,
        parameter_batch=p0.astype(complex), stop_event=stop_event, precision="mixed")
    np.testing.assert_array_equal(out.detach().cpu().numpy().reshape(-1), np.asarray(ref_vals).reshape(-1))
    o = op.options(t0=t_span[0], t1=t_span[1], abstol=1e-11, reltol=1e-8, dt=1e-3 / g,
                   saveat=None if integral else np.array([t_span[1]]), save_start=integral, maxiters=100000,
                   solver="tsit5", output=output, output_indices=None, output_when="final",
                   integral_weights=w if integral else None, stop_event=stop_event)
    steps = tape.steps()

    def replay(p):
        v = op.solve_replay(o, d["rho0_packed"], slots, p.astype(complex), steps, event_hit=hits)
        return (np.asarray(v).reshape(b, -1) * wout).sum(axis=1)

    base = replay(p0)
    # the double-precision replay of the mixed steps is within the mixed form's error of its values
    np.testing.assert_allclose(base, (out.detach().cpu().numpy().reshape(b, -1) * wout).sum(axis=1), rtol=1e-6,
                               atol=1e-6 * np.max(np.abs(base)))
    worst = 0.0
    for k in range(p0.shape[1]):
        eps = 1e-6 * np.abs(p0[:, k])
        eps[eps == 0] = 1e-6 * g
        pp, pm = p0.copy(), p0.copy()
        pp[:, k] += eps
        pm[:, k] -= eps
        fd = (replay(pp) - replay(pm)) / (2 * eps)
        natural = np.abs(base) / np.maximum(np.abs(p0[:, k]), 1e-300)
        tol = rel * np.abs(fd) + floor * natural
        assert np.all(np.abs(grad[:, k] - fd) <= tol), (k, grad[:, k], fd, tol)
        worst = max(worst, float(np.max(np.abs(grad[:, k] - fd) / np.maximum(natural, 1e-300))))
    print(f"mixed adjoint: max |grad - fd| / (|J| / |p|) = {worst:.2e}")
    return grad, worst


@pytest.mark.parametrize("output,ck", [("excited_population", 0), ("populations", 0), ("excited_population", 7),
                                       ("excited_population", 512)])
def test_mixed_form_gradients(q1, output, ck):
    """The mixed form's gradients (forward with a single-precision tape, single-precision reverse
    products): full and checkpointed tapes, integral and final populations."""
    d, plan, op = q1
    _mixed_fd_check(d, plan, op, _params(d), _slots(d), d["t_span"], output=output, checkpoint_every=ck)


@pytest.mark.parametrize("tpt", [32, 128])
def test_mixed_form_gradients_at_other_widths(q1, tpt):
    d, plan, op = q1
    plan.set_shape(tpt, 0)
    try:
        _mixed_fd_check(d, plan, op, _params(d)[:3], _slots(d), d["t_span"])
    finally:
        plan.set_shape(0, 0)


def test_mixed_form_gradients_through_a_time_event(golden):
    d = golden("plan_q1_16_tend")
    g = d["gamma"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [names.index(s) for s in ("rabi", "detuning", "theta", "t_end")]
    p0 = np.array([[1.0 * g, 0.0, 0.3, 123.4 / g], [3.0 * g, -2.0 * g, 1.1, 60.3 / g], [0.4 * g, 1.5 * g, 2.5, 250.0 / g]])
    for ck in (0, 9):
        _mixed_fd_check(d, NativePlan(d["payload"]), oracle.OraclePlan(d["payload"]), p0, slots, (0.0, 200.0 / g),
                        checkpoint_every=ck, stop_event=_t_end_event(names), hits_expected=[1, 1, 0])


@pytest.mark.parametrize("wide", [False, True])
def test_mixed_form_gradients_of_the_76_state_system(golden, monkeypatch, wide):
    """256 threads per trajectory (the sweep's buffers in device memory), checkpointed: the tight
    shape (24 elements per thread) and, with OBE_EPT_WIDE, the widest (32), which systems of 79-90
    states run."""
    if wide:
        monkeypatch.setenv("OBE_EPT_WIDE", "1")
    d = golden("plan_rc_76")
    g = d["gamma"]
    plan = NativePlan(d["payload"])
    op = oracle.OraclePlan(d["payload"])
    p0 = np.array([[1.2 * g, 2.0 * g, 0.3 * g, -0.2 * g], [2.5 * g, 0.8 * g, -0.4 * g, 0.6 * g]])
    _mixed_fd_check(d, plan, op, p0, _slots(d, ("Ω0", "Ω1", "δ0", "δ1")), (0.0, 6.0 / g), checkpoint_every=16)


def test_gradients_of_two_plans_on_concurrent_streams(golden):
    """The C-ABI gradient entry points on two plans at once, each on its own stream (taped forwards,
    one synchronisation, reverse sweeps): the same gradients as the autograd wrapper gives one plan
    at a time (per-trajectory arithmetic does not depend on the schedule)."""
    dev = torch.device("cuda", 0)
    runs = []
    for name, slot_names in (("plan_q1_16_tend", ("rabi", "detuning", "theta", "t_end")),
                             ("plan_r0_39", ("rabi", "detuning", "theta", "t_end"))):
        d = golden(name)
        g = d["gamma"]
        names = d["payload"]["parameter_graph"]["slot_names"]
        slots = [names.index(s) for s in slot_names]
        p0 = np.array([[1.5 * g, 0.5 * g, 0.4, 60.0 / g], [3.0 * g, -1.0 * g, 1.2, 45.0 / g], [0.5 * g, 2.0 * g, 2.2, 80.0 / g]])
        plan = NativePlan(d["payload"])
        w = [(i, 1.0) for i in d["excited_indices"]]
        pt = torch.tensor(p0, dtype=torch.float64, device=dev, requires_grad=True)
        out, tape = solve_batch_with_grad(plan, d["rho0_packed"], (0.0, 100.0 / g), pt, slots, dt=1e-3 / g,
                                          integral_weights=w, stop_event=_t_end_event(names), precision="mixed",
                                          return_tape=True)
        out.sum().backward()
        runs.append(dict(plan=plan, opts=tape.opts, b=3, slots=slots, ref=pt.grad, ms=tape.max_steps,
                         ck=tape.checkpoint_every, rho=tape.rho0, pv=tape.pvals, stream=torch.cuda.Stream(dev)))
    for r in runs:
        r["tape"] = torch.empty(r["b"] * r["plan"].grad_tape_doubles(r["ms"], r["ck"], "mixed"), dtype=torch.float64,
                                device=dev)
        r["stats"] = torch.zeros(r["b"] * 6, dtype=torch.int64, device=dev)
        r["out"] = torch.zeros(r["b"], dtype=torch.float64, device=dev)
        r["pg"] = torch.zeros(r["b"], len(r["slots"]), dtype=torch.float64, device=dev)
        r["ast"] = torch.zeros(r["b"], dtype=torch.int32, device=dev)
        r["og"] = torch.ones(r["b"], dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    for r in runs:
        r["plan"].grad_forward(r["opts"], r["b"], r["rho"].data_ptr(), r["slots"], r["pv"].data_ptr(), r["ms"],
                               r["tape"].data_ptr(), r["out"].data_ptr(), r["stats"].data_ptr(), r["stream"].cuda_stream,
                               checkpoint_every=r["ck"])
    torch.cuda.synchronize()
    for r in runs:
        r["plan"].grad_backward(r["opts"], r["b"], r["rho"].data_ptr(), r["slots"], r["pv"].data_ptr(), r["slots"], r["ms"],
                                r["tape"].data_ptr(), r["stats"].data_ptr(), r["og"].data_ptr(), r["pg"].data_ptr(), None,
                                r["ast"].data_ptr(), r["stream"].cuda_stream, checkpoint_every=r["ck"])
    torch.cuda.synchronize()
    for r in runs:
        assert not bool(r["ast"].any())
        assert torch.equal(r["pg"], r["ref"])
