"""torch.autograd.Function wrappers over the C-ABI's adjoint gradient.

- `rd_objective(x, ctx, d1)`: J(p, kappa, rho) of DerivativeOperatorsRD; the gradient comes from
  one forward + adjoint sweep (glia_eval_objective_and_gradient) run in the forward pass when x
  requires grad, and is replayed in backward.
- `solve_state(c0, ctx)`: the forward map c0 -> c(1) (PdeOperatorsRD::solveState). Its backward
  is the discrete adjoint: dL/dc0 = (dc1/dc0)^T g = solveAdjoint(p_t = g), the linear map the
  reference's solveAdjoint applies to its final condition (src/pde/PdeOperators.cpp:372-420).
- `phi_apply(p, ctx)`: c0 = Phi p with backward Phi^T g (stored-mode normalisation, in which
  Phi and Phi^T are exact transposes).

`ctx` is a glia_gb300.context.Context (host pointer mode); tensors may live on any device and are
moved through host float64 buffers, matching the C-ABI's default mode.
"""
from __future__ import annotations

import numpy as np
import torch


def _np(t: torch.Tensor) -> np.ndarray:
    return t.detach().to("cpu", torch.float64).contiguous().numpy()


class RDObjective(torch.autograd.Function):
    @staticmethod
    def forward(fctx, x, ctx, d1):
        xn = _np(x)
        d = _np(d1) if isinstance(d1, torch.Tensor) else np.asarray(d1, dtype=np.float64)
        if x.requires_grad:
            J, dJ = ctx.eval_objective_and_gradient(xn, d)
            fctx.save_for_backward(torch.from_numpy(dJ))
        else:
            J = ctx.eval_objective(xn, d)
            fctx.save_for_backward(torch.zeros(0, dtype=torch.float64))
        return torch.tensor(J, dtype=x.dtype, device=x.device)

    @staticmethod
    def backward(fctx, gJ):
        (dJ,) = fctx.saved_tensors
        return gJ * dJ.to(gJ.device, gJ.dtype), None, None


class SolveState(torch.autograd.Function):
    @staticmethod
    def forward(fctx, c0, ctx):
        c0n = _np(c0)
        c1 = ctx.solve_state(c0n)
        fctx.ctx = ctx
        fctx.c0 = c0n
        fctx.generation = _bump(ctx)
        return torch.from_numpy(c1).to(c0.device, c0.dtype)

    @staticmethod
    def backward(fctx, g):
        ctx = fctx.ctx
        if getattr(ctx, "_autograd_generation", None) != fctx.generation:
            # another state solve ran on this context since the forward: rebuild the history
            ctx.solve_state(fctx.c0)
            fctx.generation = _bump(ctx)
        a0 = ctx.solve_adjoint(_np(g))
        return torch.from_numpy(a0).to(g.device, g.dtype), None


class PhiApply(torch.autograd.Function):
    @staticmethod
    def forward(fctx, p, ctx):
        fctx.ctx = ctx
        fctx.np = p.numel()
        return torch.from_numpy(ctx.phi_apply(_np(p))).to(p.device, p.dtype)

    @staticmethod
    def backward(fctx, g):
        pt = fctx.ctx.phi_apply_transpose(_np(g), fctx.np)
        return torch.from_numpy(pt).to(g.device, g.dtype), None


_gen = [0]


def _bump(ctx) -> int:
    _gen[0] += 1
    ctx._autograd_generation = _gen[0]
    return _gen[0]


def rd_objective(x: torch.Tensor, ctx, d1) -> torch.Tensor:
    """J(x) with x = [p (np), kappa (nk), rho (nr)]; differentiable w.r.t. x."""
    return RDObjective.apply(x, ctx, d1)


def solve_state(c0: torch.Tensor, ctx) -> torch.Tensor:
    """c(1) from c(0); differentiable w.r.t. c(0) through the discrete adjoint."""
    return SolveState.apply(c0, ctx)


def phi_apply(p: torch.Tensor, ctx) -> torch.Tensor:
    """c0 = Phi p; differentiable w.r.t. p (set opt phi_store=1 for exact transposes)."""
    return PhiApply.apply(p, ctx)
