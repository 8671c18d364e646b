"""Differentiable batched solves: a ``torch.autograd.Function`` over the GPU solver's discrete
adjoint (obe_grad_forward / obe_grad_backward).

The reference has no gradient path (its ``lindblad_jvp_py`` is the linear RHS itself), so this
module has no counterpart there.  The forward pass is the adaptive solve, double precision or
the mixed form (single-precision RHS, double-precision state); it records every accepted step on
the device (the tape: start time, size, start state and six stage derivatives per step; the mixed
form's in single precision, and its reverse sweep runs the transposed and parameter products in
single precision with double-precision accumulation).  The backward pass is the exact adjoint of that discrete solve with the
step sequence frozen -- what central finite differences of the solve with the same steps give --
for the final weighted integral (``excited_population``, ``photon_integral``,
``weighted_integral``) or the final populations, with respect to any scalar base parameter slots
and the packed initial state.  A ``stop_event`` (population threshold or runtime expression) may
end each trajectory: the step that ends on it maps to the dense output at the event time, and the
event time's own dependence on the state and parameters enters through the event function's
derivatives.

Example::

    plan = NativePlan(payload)
    params = torch.tensor(values, dtype=torch.float64, device="cuda", requires_grad=True)  # (B, S)
    J = solve_batch_with_grad(plan, rho0, (t0, t1), params, slots, output="excited_population",
                              integral_weights=[(13, 1.0), (14, 1.0), (15, 1.0)])
    J.sum().backward()  # params.grad: dJ/dparameter per trajectory
"""

from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from . import _abi
from ._options import INTEGRAL_OUTPUTS
from .native import NativePlan

__all__ = ["solve_batch_with_grad", "ForwardTape"]

_ADJ_MESSAGES = {
    1: "a helper function or interpolation table receives an argument that depends on a differentiated parameter",
    2: "the forward trajectory failed or ran past the tape",
    3: "the stop event's function has a zero time derivative at the crossing",
}


def _precision(opts) -> str:
    """The form an options object solves in ("fp64" or "mixed")."""
    return "mixed" if int(opts.opts.precision) == _abi.PRECISIONS["mixed"] else "fp64"


class ForwardTape:
    """What the backward pass needs of a forward solve: its options, inputs, tape and statistics."""

    def __init__(self, plan: NativePlan, opts, rho0: torch.Tensor, slots: list[int], pvals: torch.Tensor,
                 max_steps: int, tape: torch.Tensor, stats: torch.Tensor, checkpoint_every: int = 0):
        self.plan, self.opts, self.rho0, self.slots, self.pvals = plan, opts, rho0, slots, pvals
        self.max_steps, self.tape, self.stats = max_steps, tape, stats
        self.checkpoint_every = checkpoint_every

    def steps(self) -> list[np.ndarray]:
        """The accepted steps (t_n, h_n) of every trajectory, as recorded."""
        st = self.stats.view(-1, 6).cpu().numpy()
        b = st.shape[0]
        prec = _precision(self.opts) if self.opts is not None else "fp64"
        if self.checkpoint_every > 0:
            per = self.plan.grad_tape_doubles(self.max_steps, self.checkpoint_every, prec)
            tape = self.tape.view(b, per)[:, : 2 * self.max_steps].reshape(b, self.max_steps, 2).cpu().numpy()
        else:
            per = self.plan.grad_tape_doubles_per_step(prec)
            tape = self.tape.view(b, self.max_steps, per)[:, :, :2].cpu().numpy()
        return [tape[k, : int(st[k, 0])] for k in range(b)]

    def event_hits(self) -> np.ndarray:
        """Per trajectory: 1 where the stop event ended the solve (its last step is the event step)."""
        st = self.stats.view(-1, 6).cpu().numpy()
        return (st[:, 3] & 0xFFFFFFFF).astype(np.int32)


def _checkpoint_every(plan: NativePlan, b: int, max_steps: int, requested: int | None, device=None,
                      precision: str = "fp64") -> int:
    """The full tape while it takes at most a quarter of the device's free memory (at least
    4 GiB), else a start state every 512 steps."""
    if requested is not None:
        return int(requested)
    budget = 4 << 30
    if device is not None and device.type == "cuda":
        budget = max(budget, torch.cuda.mem_get_info(device)[0] // 4)
    return 0 if b * plan.grad_tape_doubles(max_steps, 0, precision) * 8 <= budget else 512


def _forward(plan: NativePlan, opts, rho0: torch.Tensor, slots: list[int], pvals: torch.Tensor, max_steps: int,
             checkpoint_every: int | None = None):
    b = rho0.shape[0]
    stream = torch.cuda.current_stream(rho0.device).cuda_stream
    while True:
        prec = _precision(opts)
        ck = _checkpoint_every(plan, b, max_steps, checkpoint_every, rho0.device, prec)
        tape = torch.empty(b * plan.grad_tape_doubles(max_steps, ck, prec), dtype=torch.float64, device=rho0.device)
        values = torch.empty(b * opts.width, dtype=torch.float64, device=rho0.device)
        stats = torch.zeros(b * 6, dtype=torch.int64, device=rho0.device)
        plan.grad_forward(opts, b, rho0.data_ptr(), slots, pvals.data_ptr() if slots else None, max_steps,
                          tape.data_ptr(), values.data_ptr(), stats.data_ptr(), stream, checkpoint_every=ck)
        st = stats.view(b, 6).cpu().numpy()
        status = st[:, 3] >> 32
        if np.all(status == 0):
            return values.view(b, opts.width), ForwardTape(plan, opts, rho0, slots, pvals, max_steps, tape, stats, ck)
        if int(st[:, 0].max()) < max_steps:
            bad = int(np.flatnonzero(status != 0)[0])
            raise ValueError(f"trajectory {bad}: the forward solve failed (status {int(status[bad])})")
        max_steps *= 2  # the tape was too short: record again with twice the room


class _SolveWithGrad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor, rho0: torch.Tensor, plan: NativePlan, opts, slots: list[int], max_steps: int,
                checkpoint_every):
        b = rho0.shape[0]
        pvals = torch.zeros(b, len(slots), 2, dtype=torch.float64, device=rho0.device)
        if slots:
            pvals[:, :, 0] = params.detach()
        pvals = pvals.contiguous()
        values, tape = _forward(plan, opts, rho0.detach().contiguous(), slots, pvals, max_steps, checkpoint_every)
        ctx.tape = tape
        return values.squeeze(1) if opts.width == 1 else values

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        t: ForwardTape = ctx.tape
        b = t.rho0.shape[0]
        n_grad = len(t.slots)
        dev = t.rho0.device
        g = grad_out.detach().to(torch.float64).contiguous().view(b, -1)
        pgrad = torch.zeros(b, max(n_grad, 1), dtype=torch.float64, device=dev)
        rgrad = torch.zeros(b, t.rho0.shape[1], dtype=torch.float64, device=dev) if ctx.needs_input_grad[1] else None
        status = torch.zeros(b, dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        t.plan.grad_backward(t.opts, b, t.rho0.data_ptr(), t.slots, t.pvals.data_ptr() if t.slots else None, t.slots,
                             t.max_steps, t.tape.data_ptr(), t.stats.data_ptr(), g.data_ptr(),
                             pgrad.data_ptr() if n_grad else None, rgrad.data_ptr() if rgrad is not None else None,
                             status.data_ptr(), stream, checkpoint_every=t.checkpoint_every)
        st = status.cpu().numpy()
        if np.any(st != 0):
            bad = int(np.flatnonzero(st != 0)[0])
            raise ValueError(f"trajectory {bad}: gradient not available: {_ADJ_MESSAGES.get(int(st[bad]), int(st[bad]))}")
        return (pgrad[:, :n_grad] if n_grad else None), rgrad, None, None, None, None, None


def solve_batch_with_grad(plan: NativePlan, rho0, t_span: Sequence[float], params: torch.Tensor,
                          parameter_slot_indices: Sequence[int], *, solver: str = "tsit5", abstol: float = 1e-11,
                          reltol: float = 1e-8, dt: float = 0.0, maxiters: int = 100000,
                          output: str = "excited_population", integral_weights=None, max_steps: int = 4096,
                          checkpoint_every: int | None = None, stop_event=None, precision: str = "fp64",
                          return_tape: bool = False):
    """Batched double-precision solve whose outputs are differentiable in ``params`` ((B, S) real,
    the values of the base slots ``parameter_slot_indices``) and in ``rho0`` ((B, N) packed).

    ``output``: a weighted integral (final value, shape (B,)) or ``"populations"`` (final
    populations, shape (B, n)).  ``max_steps`` sizes the tape (doubled and retried on overflow).
    ``checkpoint_every``: 0 records every step's stage derivatives; C > 0 records the start state
    of every C-th step and the reverse sweep recomputes each segment from it (one more forward's
    work, a tape of 2 + N / C doubles per step); None takes the full tape while it fits in a
    quarter of the device's free memory.  ``stop_event``: as in the solves (``{"kind": "population", "indices", "threshold"}`` or
    ``{"kind": "runtime_expression", "expression"}``); the outputs end at the event time.
    ``precision``: ``"fp64"`` or ``"mixed"`` (the forward and the reverse sweep in the mixed form).
    With ``return_tape`` the forward tape comes back too (its ``steps()`` are the frozen steps,
    its ``event_hits()`` which trajectories ended on the event).
    """
    t0, t1 = float(t_span[0]), float(t_span[1])
    if output in INTEGRAL_OUTPUTS:
        opts = plan.options(t0=t0, t1=t1, abstol=abstol, reltol=reltol, dt=dt, saveat=None, save_start=True,
                            maxiters=maxiters, solver=solver, output=output, output_indices=None, output_when="final",
                            integral_weights=integral_weights, stop_event=stop_event, precision=precision)
    elif output == "populations":
        opts = plan.options(t0=t0, t1=t1, abstol=abstol, reltol=reltol, dt=dt, saveat=np.array([t1]), save_start=False,
                            maxiters=maxiters, solver=solver, output="populations", output_indices=None,
                            output_when="final", integral_weights=None, stop_event=stop_event, precision=precision)
    else:
        raise NotImplementedError("gradients are available for final weighted integrals and final populations")
    dev = params.device
    if not torch.is_tensor(rho0):
        rho0 = torch.as_tensor(np.asarray(rho0, dtype=np.float64), device=dev)
    rho0 = rho0.to(device=dev, dtype=torch.float64)
    params = params.to(dtype=torch.float64)
    if rho0.dim() == 1:
        rho0 = rho0.unsqueeze(0).expand(params.shape[0], -1)
    slots = [int(s) for s in parameter_slot_indices]
    out = _SolveWithGrad.apply(params, rho0.contiguous(), plan, opts, slots, int(max_steps), checkpoint_every)
    if return_tape:
        return out, out.grad_fn.tape if out.grad_fn is not None else None
    return out
