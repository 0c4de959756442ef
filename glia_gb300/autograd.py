"""torch.autograd.Function wrappers over the C-ABI's adjoint gradient.

- `rd_objective(x, ctx, d1)`: J(p, kappa, rho) of DerivativeOperatorsRD; the gradient comes from
  one forward + adjoint sweep (glia_eval_objective_and_gradient) run in the forward pass when x
  requires grad, and is replayed in backward.
- `solve_state(c0, ctx)`: the forward map c0 -> c(1) (PdeOperatorsRD::solveState). Its backward
  is the discrete adjoint: dL/dc0 = (dc1/dc0)^T g = solveAdjoint(p_t = g), the linear map the
  reference's solveAdjoint applies to its final condition (src/pde/PdeOperators.cpp:372-420).
- `phi_apply(p, ctx)`: c0 = Phi p with backward Phi^T g (stored-mode normalisation, in which
  Phi and Phi^T are exact transposes).

`ctx` is a glia_gb300.context.Context. Grid fields that are CUDA tensors of float64 or float32
go to the library as device pointers (GLIA_PTR_DEVICE_F64 / _F32) on the caller's current torch
stream, with no host round trip; other tensors (CPU, other dtypes) go through host float64
buffers. Parameter vectors (x, p) are always host float64, as in the C-ABI.

A backward that needs the state history checks `Context.generation`, which every call that
rewrites the history, the coefficients or the model settings advances: if anything ran on the
context since the forward, the forward solve is repeated before the adjoint.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _abi


def _np(t: torch.Tensor) -> np.ndarray:
    return t.detach().to("cpu", torch.float64).contiguous().numpy()


class _FieldCall:
    """Pointer mode and stream of one library call whose grid fields are shaped like `like`
    (a tensor, or a (device, dtype, shape) triple)."""

    _MODES = {torch.float64: _abi.GLIA_PTR_DEVICE_F64, torch.float32: _abi.GLIA_PTR_DEVICE_F32}

    def __init__(self, ctx, like):
        self.ctx = ctx
        if isinstance(like, torch.Tensor):
            self.dev, self.dtype, self.shape = like.device, like.dtype, like.shape
        elif isinstance(like, tuple):
            self.dev, self.dtype, self.shape = like
        else:  # host array
            self.dev, self.dtype, self.shape = torch.device("cpu"), torch.float64, (ctx.N,)
        self.device = self.dev.type == "cuda" and self.dtype in self._MODES

    def __enter__(self):
        if self.device:
            self.mode0, self.stream0 = self.ctx.ptr_mode, self.ctx.stream
            self.ctx.set_pointer_mode(self._MODES[self.dtype])
            self.ctx.set_stream(torch.cuda.current_stream(self.dev).cuda_stream)
        return self

    def __exit__(self, *exc):
        if self.device:
            self.ctx.set_pointer_mode(self.mode0)
            self.ctx.set_stream(self.stream0)

    def inp(self, t):
        """A grid field argument (tensor or array) in this call's pointer mode."""
        if self.device:
            if not isinstance(t, torch.Tensor):
                t = torch.as_tensor(np.asarray(t))
            return t.detach().to(self.dev, self.dtype).contiguous().view(-1)
        return _np(t) if isinstance(t, torch.Tensor) else np.asarray(t, dtype=np.float64)

    def out(self):
        if self.device:
            return torch.empty(self.ctx.N, dtype=self.dtype, device=self.dev)
        return None

    def result(self, r):
        if self.device:
            return r.view(self.shape)
        return torch.from_numpy(r).to(self.dev, self.dtype).view(self.shape)


class RDObjective(torch.autograd.Function):
    @staticmethod
    def forward(fctx, x, ctx, d1):
        xn = _np(x)
        with _FieldCall(ctx, d1) as fc:
            d = fc.inp(d1)
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
        with _FieldCall(ctx, c0) as fc:
            c1 = ctx.solve_state(fc.inp(c0), out=fc.out())
            out = fc.result(c1)
        fctx.ctx = ctx
        fctx.save_for_backward(c0.detach().clone())
        fctx.generation = ctx.generation
        return out

    @staticmethod
    def backward(fctx, g):
        ctx = fctx.ctx
        (c0,) = fctx.saved_tensors
        with _FieldCall(ctx, g) as fc:
            if ctx.generation != fctx.generation:
                # the history was rewritten since the forward: rebuild it from c(0)
                ctx.solve_state(fc.inp(c0), out=fc.out())
                fctx.generation = ctx.generation
            a0 = ctx.solve_adjoint(fc.inp(g), out=fc.out())
            return fc.result(a0), None


class PhiApply(torch.autograd.Function):
    @staticmethod
    def forward(fctx, p, ctx, like):
        fctx.ctx = ctx
        fctx.np = p.numel()
        fctx.p_like = (p.device, p.dtype)
        fctx.phi_generation = ctx.phi_generation
        with _FieldCall(ctx, like) as fc:
            return fc.result(ctx.phi_apply(_np(p), out=fc.out()))

    @staticmethod
    def backward(fctx, g):
        ctx = fctx.ctx
        if ctx.phi_generation != fctx.phi_generation:
            raise RuntimeError("phi_apply backward: the basis (set_phi / set_opt / set_tissue) "
                               "changed since the forward")
        with _FieldCall(ctx, g) as fc:
            pt = ctx.phi_apply_transpose(fc.inp(g), fctx.np)
        dev, dtype = fctx.p_like
        return torch.from_numpy(pt).to(dev, dtype), None, None


def rd_objective(x: torch.Tensor, ctx, d1) -> torch.Tensor:
    """J(x) with x = [p (np), kappa (nk), rho (nr)]; differentiable w.r.t. x. `d1` may be a CUDA
    tensor (device path) or a host array."""
    return RDObjective.apply(x, ctx, d1)


def solve_state(c0: torch.Tensor, ctx) -> torch.Tensor:
    """c(1) from c(0); differentiable w.r.t. c(0) through the discrete adjoint."""
    return SolveState.apply(c0, ctx)


def phi_apply(p: torch.Tensor, ctx, device=None) -> torch.Tensor:
    """c0 = Phi p; differentiable w.r.t. p (set opt phi_store=1 for exact transposes). The
    field comes back on `device` (default p's device) in p's dtype (float64 unless p is
    float32)."""
    dev = torch.device(device) if device is not None else p.device
    dtype = p.dtype if p.dtype in (torch.float32, torch.float64) else torch.float64
    return PhiApply.apply(p, ctx, (dev, dtype, (ctx.N,)))
