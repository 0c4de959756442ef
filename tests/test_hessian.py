"""Gauss-Newton Hessian matvec (DerivativeOperatorsRD::evaluateHessian, p block) and the
linearised solves it is made of (solveState(1), solveAdjoint(2)).

CPU tests run on the FP64 oracle: linearity, the finite-difference derivative of the gradient at
a zero residual, the call-order error. GPU tests compare the CUDA library with the oracle in every
engine / precision and check checkpointed == full history."""
import numpy as np
import pytest

from glia_gb300 import _abi
from tests.helpers import rel_l2


def _problem(ctx_factory, n=32, nt=4, n_gauss=8, history=_abi.GLIA_HISTORY_FULL, every=2):
    from tests.gpu_common import configure, small_problem

    wl, tissue, centers = small_problem(n, nt, n_gauss=n_gauss)
    ctx = ctx_factory(n)
    configure(ctx, wl, tissue, centers, history, every)
    ctx.set_opt(diffusivity_inversion=0, all_gradients=0, flag_reaction_inv=0)
    ctx.set_obs_filter(np.ones(n ** 3))
    rng = np.random.default_rng(7)
    p = rng.uniform(0.2, 0.9, n_gauss)
    x = np.concatenate([p, [wl.kappa, wl.rho]])
    return ctx, wl, x, rng


def _orc(n):
    from oracle import oracle

    return oracle.context(n)


def test_oracle_linearised_state_needs_a_state_solve():
    ctx, wl, x, _ = _problem(_orc)
    with pytest.raises(RuntimeError):
        ctx.solve_state(np.zeros(wl.n ** 3), linearized=1)


def test_oracle_hessian_is_linear_and_matches_gradient_differences():
    ctx, wl, x, rng = _problem(_orc)
    ctx.set_pcg(1e-10, 5000, 1, wl.dt)
    np_ = len(x) - 2
    d = ctx.solve_state(ctx.phi_apply(x[:np_]))  # zero residual at x: GN = exact Hessian
    J, g0 = ctx.eval_objective_and_gradient(x, d)
    assert J < 1e-12
    u = np.concatenate([rng.standard_normal(np_), [0.0, 0.0]])
    v = np.concatenate([rng.standard_normal(np_), [0.0, 0.0]])
    Hu = ctx.hessian_matvec(u)
    Hv = ctx.hessian_matvec(v)
    Huv = ctx.hessian_matvec(2.0 * u - 0.5 * v)
    assert rel_l2(Huv, 2.0 * Hu - 0.5 * Hv) < 1e-8
    assert np.all(Hu[np_:] == 0.0)
    # derivative of the gradient along u (dense p keeps the on-the-fly normalisation fixed); the
    # reference linearises the logistic step at the state of the step's start rather than at
    # the half step, an O(dt) difference
    eps = 1e-3
    gp = ctx.eval_gradient(x + eps * u, d)
    gm = ctx.eval_gradient(x - eps * u, d)
    fd = (gp - gm)[:np_] / (2 * eps)
    assert rel_l2(Hu[:np_], fd) < 2e-3
    # <u, H u> > 0 (GN Hessian is positive semi-definite up to that difference)
    assert u[:np_] @ Hu[:np_] > 0


def test_oracle_hessian_l2b_regulariser():
    ctx, wl, x, rng = _problem(_orc)
    ctx.set_opt(regularization_norm=1, beta=0.25)
    np_ = len(x) - 2
    d = ctx.solve_state(ctx.phi_apply(x[:np_]))
    ctx.eval_objective_and_gradient(x, d)
    u = np.concatenate([rng.standard_normal(np_), [0.3, -0.2]])
    Hu = ctx.hessian_matvec(u)
    ctx.set_opt(beta=0.0)
    ctx.eval_objective_and_gradient(x, d)
    Hu0 = ctx.hessian_matvec(u)
    assert rel_l2(Hu - Hu0, 0.25 * u) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision,engine,tol", [
    (_abi.GLIA_FP64, _abi.GLIA_ENGINE_FUSED, 1e-9),
    (_abi.GLIA_FP64, _abi.GLIA_ENGINE_REFERENCE, 1e-9),
    (_abi.GLIA_MIXED, _abi.GLIA_ENGINE_FUSED, 1e-4),
])
def test_gpu_hessian_matches_oracle(precision, engine, tol):
    from tests.gpu_common import gpu

    n = 32
    octx, wl, x, rng = _problem(_orc, n)
    gctx, _, _, _ = _problem(lambda m: gpu(m, precision, engine), n)
    np_ = len(x) - 2
    d = octx.solve_state(octx.phi_apply(0.8 * x[:np_]))
    u = np.concatenate([rng.standard_normal(np_), [0.0, 0.0]])
    octx.eval_objective_and_gradient(x, d)
    gctx.eval_objective_and_gradient(x, d)
    assert rel_l2(gctx.hessian_matvec(u), octx.hessian_matvec(u)) < tol
    # the linearised forward on its own
    c_t = octx.phi_apply(u[:np_])
    assert rel_l2(gctx.solve_state(c_t, linearized=1), octx.solve_state(c_t, linearized=1)) < tol


@pytest.mark.gpu
def test_gpu_hessian_checkpointed_equals_full_history():
    from tests.gpu_common import gpu

    n = 32
    full, wl, x, rng = _problem(lambda m: gpu(m, _abi.GLIA_MIXED), n, nt=6)
    ckpt, _, _, _ = _problem(lambda m: gpu(m, _abi.GLIA_MIXED), n, nt=6,
                             history=_abi.GLIA_HISTORY_CHECKPOINT, every=4)
    np_ = len(x) - 2
    d = full.solve_state(full.phi_apply(0.7 * x[:np_]))
    u = np.concatenate([rng.standard_normal(np_), [0.0, 0.0]])
    full.eval_objective_and_gradient(x, d)
    ckpt.eval_objective_and_gradient(x, d)
    assert np.array_equal(full.hessian_matvec(u), ckpt.hessian_matvec(u))
