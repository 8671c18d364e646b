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
