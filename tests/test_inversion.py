"""Bounded L-BFGS inversion driver (glia_gb300/inversion.py): the optimiser on an analytic
bound-constrained quadratic, and a small reconstruction on a context of the FP64 oracle."""
import numpy as np
import pytest

from glia_gb300.inversion import LbfgsSettings, bounded_lbfgs, invert, reference_bounds


def test_bounded_lbfgs_on_a_bound_constrained_quadratic():
    rng = np.random.default_rng(0)
    A = rng.standard_normal((6, 6))
    H = A @ A.T + 6 * np.eye(6)
    b = rng.standard_normal(6)
    lb, ub = np.full(6, -0.1), np.full(6, 0.2)

    def fg(x):
        return 0.5 * x @ H @ x - b @ x, H @ x - b

    res = bounded_lbfgs(fg, lambda x: fg(x)[0], np.zeros(6), lb, ub,
                        LbfgsSettings(gttol=1e-10, gatol=1e-12, maxit=200))
    # KKT: projected gradient vanishes, solution inside the box
    assert res.gnorm < 1e-8
    assert np.all(res.x >= lb - 1e-15) and np.all(res.x <= ub + 1e-15)


def test_small_reconstruction_on_the_oracle():
    from oracle import oracle
    from tests.gpu_common import configure, small_problem

    n, nt = 32, 3
    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    ctx = oracle.context(n)
    configure(ctx, wl, tissue, centers)
    ctx.set_obs_filter(np.ones(n ** 3))
    ctx.set_pcg(1e-8, 5000, 1, wl.dt)
    x_true = np.concatenate([[0.0, 0.9, 0.0, 0.0, 0.6, 0.0, 0.0, 0.0], [wl.kappa, wl.rho]])
    ctx.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    d = ctx.solve_state(ctx.phi_apply(x_true[:8]))
    lb, ub = reference_bounds(8)
    x0 = np.concatenate([np.zeros(8), [0.7 * wl.kappa, 0.8 * wl.rho]])
    res = invert(ctx, d, x0, lb, ub, LbfgsSettings(maxit=25))
    J0 = ctx.eval_objective(x0, d)
    assert res.J < 1e-3 * J0
    assert res.gnorm < 1e-2 * res.gnorm0
    assert np.linalg.norm(res.x[:8] - x_true[:8]) < 0.1 * np.linalg.norm(x_true[:8])
