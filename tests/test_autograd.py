"""The torch.autograd.Function wrappers (glia_gb300/autograd.py) on a context of the FP64
oracle (CPU, small grid) — the same Context interface the CUDA library exposes — and on the
CUDA library (GPU tests)."""
import numpy as np
import pytest
import torch

from glia_gb300 import autograd as ga
from oracle import oracle
from tests.gpu_common import configure, observation, small_problem


def _ctx(n=32, nt=2, n_gauss=4, phi_store=1, rtol=1e-11):
    wl, tissue, centers = small_problem(n, nt, n_gauss)
    ctx = oracle.context(n)
    configure(ctx, wl, tissue, centers)
    ctx.set_opt(phi_store=phi_store)
    ctx.set_obs_filter(np.ones(n ** 3))
    ctx.set_pcg(rtol, 5000, 1, wl.dt)  # fixed PC dt: results independent of call history
    return ctx, wl, tissue, centers


def test_objective_backward_is_the_adjoint_gradient():
    ctx, wl, tissue, centers = _ctx()
    d1 = observation(wl, tissue, centers)
    x = torch.tensor(np.concatenate([[0.3, 0.0, 0.7, 0.2], [wl.kappa, wl.rho]]),
                     requires_grad=True)
    J = ga.rd_objective(x, ctx, d1)
    J.backward()
    J_ref, g_ref = ctx.eval_objective_and_gradient(x.detach().numpy(), d1)
    assert J.item() == pytest.approx(J_ref, rel=1e-14)
    assert np.allclose(x.grad.numpy(), g_ref, rtol=1e-13, atol=0)


def test_solve_state_backward_is_the_transpose_of_the_forward_map():
    """<g, (dc1/dc0) v> (central differences) == <(dc1/dc0)^T g, v> (adjoint backward)."""
    ctx, wl, tissue, centers = _ctx()
    n = 32
    rng = np.random.default_rng(0)
    c0 = torch.tensor(ctx.phi_apply(np.array([0.5, 0.2, 0.0, 0.9])), requires_grad=True)
    g = torch.tensor(rng.standard_normal(n ** 3))
    c1 = ga.solve_state(c0, ctx)
    (c1 * g).sum().backward()
    v = rng.standard_normal(n ** 3) * 1e-2
    h = 1e-4
    cp = ctx.solve_state(c0.detach().numpy() + h * v)
    cm = ctx.solve_state(c0.detach().numpy() - h * v)
    lhs = float(g.numpy() @ ((cp - cm) / (2 * h)))
    rhs = float(c0.grad.numpy() @ v)
    assert lhs == pytest.approx(rhs, rel=1e-6)


def test_phi_backward_is_phi_transpose():
    ctx, *_ = _ctx()
    p = torch.tensor([0.3, 0.1, 0.0, 0.8], dtype=torch.float64, requires_grad=True)
    v = torch.tensor(np.random.default_rng(1).standard_normal(32 ** 3))
    (ga.phi_apply(p, ctx) * v).sum().backward()
    c = ctx.phi_apply(np.eye(4)[2])
    assert float(p.grad[2]) == pytest.approx(float(c @ v.numpy()), rel=1e-12)


def test_solve_state_backward_after_other_calls_on_the_context():
    """A gradient evaluation (and a coefficient change and back) between the forward and the
    backward of solve_state rewrites the context's state history; the backward must still be
    the adjoint around the forward's own states."""
    ctx, wl, tissue, centers = _ctx(nt=3)
    n = 32
    rng = np.random.default_rng(2)
    g = torch.tensor(rng.standard_normal(n ** 3))
    c0_np = ctx.phi_apply(np.array([0.6, 0.0, 0.3, 0.9]))

    c0 = torch.tensor(c0_np, requires_grad=True)
    (ga.solve_state(c0, ctx) * g).sum().backward()
    clean = c0.grad.clone()

    c0 = torch.tensor(c0_np, requires_grad=True)
    c1 = ga.solve_state(c0, ctx)
    d1 = observation(wl, tissue, centers)
    x = torch.tensor(np.concatenate([[0.9, 0.9, 0.9, 0.9], [wl.kappa, wl.rho]]),
                     requires_grad=True)
    ga.rd_objective(x, ctx, d1).backward()          # another forward + adjoint sweep
    ctx.set_coefficients(k=wl.kappa * 3, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    ctx.solve_state(c0_np * 0.5)
    ctx.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    (c1 * g).sum().backward()
    assert np.array_equal(c0.grad.numpy(), clean.numpy())


def test_context_generation_advances_on_history_writes_only():
    ctx, wl, *_ = _ctx(nt=2)
    g0 = ctx.generation
    ctx.stats()
    ctx.phi_apply(np.array([0.1, 0.2, 0.3, 0.4]))
    assert ctx.generation == g0
    ctx.solve_state(ctx.phi_apply(np.array([0.1, 0.2, 0.3, 0.4])))
    assert ctx.generation == g0 + 1
    p0 = ctx.phi_generation
    ctx.set_coefficients(k=wl.kappa, rho=wl.rho)
    assert ctx.phi_generation == p0 and ctx.generation == g0 + 2
    ctx.set_opt(phi_store=1)
    assert ctx.phi_generation == p0 + 1


def test_phi_backward_refuses_a_changed_basis():
    ctx, *_ = _ctx()
    p = torch.tensor([0.3, 0.1, 0.0, 0.8], dtype=torch.float64, requires_grad=True)
    c = ga.phi_apply(p, ctx)
    ctx.set_opt(phi_store=0)
    with pytest.raises(RuntimeError, match="changed since the forward"):
        c.sum().backward()
