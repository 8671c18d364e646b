"""Host-side logic of the differentiable solve (centrex_tlf_gb300.autograd), no GPU: the tape-size
rule, the tape readers (steps and event hits from the forward's statistics) and the option
checks that run before any device work."""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from centrex_tlf_gb300 import autograd  # noqa: E402
from centrex_tlf_gb300._abi import TRAJ_STATS_DTYPE  # noqa: E402
from centrex_tlf_gb300.native import NativePlan  # noqa: E402


class _FakePlan:
    """grad_tape_doubles of a plan with N packed reals: 2 + 7N per step in full, else the step
    log plus every C-th start state (the C ABI's obe_grad_tape_doubles)."""

    def __init__(self, N):
        self.N = N

    def grad_tape_doubles_per_step(self, precision="fp64"):
        return 2 + (4 if precision == "mixed" else 7) * self.N

    def grad_tape_doubles(self, max_steps, checkpoint_every=0, precision="fp64"):
        if checkpoint_every == 0:
            return max_steps * self.grad_tape_doubles_per_step(precision)
        return 2 * max_steps + -(-max_steps // checkpoint_every) * self.N


def test_tape_size_rule():
    plan = _FakePlan(256)
    # a requested interval wins
    assert autograd._checkpoint_every(plan, 10, 100, 7) == 7
    assert autograd._checkpoint_every(plan, 10, 100, 0) == 0
    # without a device the full tape is kept up to 4 GiB
    per_traj = plan.grad_tape_doubles(2048, 0) * 8
    fits = (4 << 30) // per_traj
    assert autograd._checkpoint_every(plan, fits, 2048, None) == 0
    assert autograd._checkpoint_every(plan, fits + 1, 2048, None) == 512
    assert autograd._checkpoint_every(plan, 1, 2048, None, torch.device("cpu")) == 0


def _stats(rows):
    st = np.zeros(len(rows), dtype=TRAJ_STATS_DTYPE)
    for k, (acc, hit, status, te) in enumerate(rows):
        st[k]["accepted_steps"] = acc
        st[k]["event_triggered"] = hit
        st[k]["status"] = status
        st[k]["event_time"] = te
    return torch.from_numpy(st.view(np.int64).copy())


def test_tape_readers_full_and_checkpointed():
    plan = _FakePlan(4)
    max_steps = 5
    stats = _stats([(3, 1, 0, 0.25), (5, 0, 0, np.nan)])
    # full tape: [traj][max_steps][2 + 7N], (t_n, h_n) first
    per = plan.grad_tape_doubles_per_step()
    full = np.zeros((2, max_steps, per))
    full[:, :, 0] = np.arange(max_steps) * 0.1
    full[:, :, 1] = 0.1
    t = autograd.ForwardTape(plan, None, torch.zeros(2, 16), [], None, max_steps, torch.from_numpy(full.reshape(-1)), stats, 0)
    steps = t.steps()
    assert [len(s) for s in steps] == [3, 5]
    np.testing.assert_allclose(steps[1][:, 0], np.arange(5) * 0.1)
    assert t.event_hits().tolist() == [1, 0]
    # checkpointed: [traj][step log 2 * max_steps | start states]
    ck = 2
    per_ck = plan.grad_tape_doubles(max_steps, ck)
    tape = np.zeros((2, per_ck))
    tape[:, : 2 * max_steps] = np.stack([np.arange(max_steps) * 0.2, np.full(max_steps, 0.2)], axis=1).reshape(-1)
    t = autograd.ForwardTape(plan, None, torch.zeros(2, 16), [], None, max_steps, torch.from_numpy(tape.reshape(-1)), stats, ck)
    steps = t.steps()
    assert [len(s) for s in steps] == [3, 5]
    np.testing.assert_allclose(steps[0][:, 0], [0.0, 0.2, 0.4])
    np.testing.assert_allclose(steps[0][:, 1], 0.2)


def test_unsupported_outputs_are_refused_before_device_work(golden):
    d = golden("plan_q1_16")
    plan = NativePlan(d["payload"])
    names = d["payload"]["parameter_graph"]["slot_names"]
    p = torch.tensor([[d["gamma"]]], dtype=torch.float64)
    for output in ("selected", "full", "rates"):
        with pytest.raises(NotImplementedError, match="final weighted integrals and final populations"):
            autograd.solve_batch_with_grad(plan, d["rho0_packed"], d["t_span"], p, [names.index("rabi")], output=output)


def test_tape_sizes_of_the_two_forms(golden):
    """The C ABI's tape sizes: the mixed form's full records are single precision (2 + 4N doubles
    of room, 16-byte aligned), its checkpointed tape is the double-precision one."""
    d = golden("plan_q1_16")
    plan = NativePlan(d["payload"])
    n2 = d["payload"]["n_states"] ** 2
    assert plan.grad_tape_doubles_per_step() == 2 + 7 * n2
    assert plan.grad_tape_doubles_per_step("mixed") == 2 + 4 * n2
    assert plan.grad_tape_doubles(100, 0, "mixed") == 100 * (2 + 4 * n2)
    assert plan.grad_tape_doubles(100, 16, "mixed") == plan.grad_tape_doubles(100, 16)
    assert plan.lib.obe_grad_tape_doubles(plan.handle, 100, 0) == 100 * (2 + 7 * n2)


def test_gradient_entry_points_refuse_unsupported_forms_on_the_host(golden):
    """obe_grad_forward's checks run before any device work: fixed-step solvers, plans wider than
    256 threads per trajectory and effective-Hamiltonian plans are refused with their messages.
    (The tape pointer is a placeholder that the refused calls never reach.)"""
    d = golden("plan_q1_16")
    plan = NativePlan(d["payload"])
    t0, t1 = d["t_span"]

    def opts(pl, **kw):
        base = dict(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / d["gamma"], saveat=None, save_start=True,
                    maxiters=1000, solver="tsit5", output="excited_population", output_indices=None, output_when="final",
                    integral_weights=[(13, 1.0)], stop_event=None)
        base.update(kw)
        return pl.options(**base)

    with pytest.raises(NotImplementedError, match="adaptive solvers 'dopri5' and 'tsit5'"):
        plan.grad_forward(opts(plan, solver="fixed_rk4"), 1, 0, [], None, 10, 16, 0, 0)
    with pytest.raises(NotImplementedError, match="final weighted integrals"):
        plan.grad_forward(opts(plan, output="populations", saveat=np.array([t1 / 2]), integral_weights=None), 1, 0, [],
                          None, 10, 16, 0, 0)
    big = NativePlan(golden("plan_rc_76")["payload"])
    big.set_shape(512, 0)
    with pytest.raises(NotImplementedError, match="256 threads per trajectory or fewer"):
        big.grad_forward(opts(big, integral_weights=[(70, 1.0)]), 1, 0, [], None, 10, 16, 0, 0)
    eff = NativePlan.from_effective(golden("plan_eff_r0")["plan"])
    with pytest.raises(NotImplementedError, match="expanded_sparse plans"):
        eff.grad_forward(eff.options(t0=0.0, t1=1e-6, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=None, save_start=True,
                                     maxiters=1000, solver="tsit5", output="photon_integral", output_indices=None,
                                     output_when="final", integral_weights=[(0, 1.0)], stop_event=None),
                         1, 0, [], None, 10, 16, 0, 0)
