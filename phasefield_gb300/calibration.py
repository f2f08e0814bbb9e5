"""Calibration harness: the step's hand-written adjoint as a torch.autograd.Function.

Only the calibration and test harness uses torch here; the forward and the
reverse sweep both run in libpfstep (pf_adj_*).  The differentiable input is
the vector of scale factors s = (interface mobility, interface energy, D_C,
D_Mn) applied to the model's parameters; the output is the chosen objective at
the end of ``nsteps`` steps (0: mean ferrite fraction, 1: mean austenite
carbon).  Time step and sub-step count stay those of s = 1.

    # checkpoint_every=0: record mode (the trajectory kept in HBM, no
    # recomputation); a positive interval when it does not fit
    A = phasefield_gb300.Adjoint(model, PF_PREC_FP32C, checkpoint_every=0)
    A.upload(state, 0.0)
    s = torch.ones(4, dtype=torch.float64, requires_grad=True)
    J = StepObjective.apply(s, A, 2000, 1)
    J.backward()          # s.grad = dJ/ds from the adjoint
"""
from __future__ import annotations

import numpy as np


def _torch():
    import torch

    return torch


class _Fn:
    """Built lazily so importing this module does not need torch."""

    cls = None


def step_objective():
    if _Fn.cls is not None:
        return _Fn.cls
    torch = _torch()

    class StepObjective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, scales, adjoint, nsteps: int, objective: int):
            s = scales.detach().cpu().double().numpy()
            adjoint.set_scales(s)
            J = adjoint.forward(int(nsteps))
            ctx.adjoint = adjoint
            ctx.objective = int(objective)
            return scales.new_tensor(float(J[int(objective)]))

        @staticmethod
        def backward(ctx, grad_out):
            g = ctx.adjoint.gradient(ctx.objective)
            grad = grad_out.detach().cpu().double() * _torch().from_numpy(np.asarray(g, np.float64))
            return grad.to(grad_out.dtype), None, None, None

    _Fn.cls = StepObjective
    return StepObjective


def objective(scales, adjoint, nsteps: int, objective: int):
    """J(s) with the adjoint as its backward."""
    return step_objective().apply(scales, adjoint, nsteps, objective)
