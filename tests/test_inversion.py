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


def test_more_thuente_meets_the_strong_wolfe_conditions():
    """The first test function of More and Thuente (1994), phi(a) = -a / (a^2 + beta), beta = 2,
    from four starting steps: each returned step satisfies sufficient decrease and the curvature
    condition with ftol = 1e-3, gtol = 0.1 (their Table 1 settings)."""
    from glia_gb300.inversion import more_thuente

    beta = 2.0

    def phi(a):
        f = -a / (a * a + beta)
        g = (a * a - beta) / (a * a + beta) ** 2
        return f, g, a

    s = LbfgsSettings(mt_ftol=1e-3, mt_gtol=0.1, ls_max_funcs=30)
    f0, g0 = phi(0.0)[:2]
    for a0 in (1e-3, 1e-1, 1e1, 1e3):
        t, f, payload, nfev, ok = more_thuente(phi, f0, g0, a0, s)
        assert ok and payload == t
        assert f <= f0 + 1e-3 * t * g0
        assert abs(phi(t)[1]) <= 0.1 * abs(g0)
        assert nfev <= 12


@pytest.mark.parametrize("line_search", ["mt", "armijo"])
@pytest.mark.parametrize("scale_type", ["none", "scalar", "diagonal"])
def test_bounded_lbfgs_options_reach_the_kkt_point(line_search, scale_type):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((8, 8))
    H = A @ A.T + np.diag(np.linspace(1, 50, 8))   # badly scaled: the diagonal scaling helps
    b = rng.standard_normal(8) * 5
    lb, ub = np.full(8, -0.2), np.full(8, 0.3)

    def fg(x):
        return 0.5 * x @ H @ x - b @ x, H @ x - b

    res = bounded_lbfgs(fg, lambda x: fg(x)[0], np.zeros(8), lb, ub,
                        LbfgsSettings(gttol=1e-10, gatol=1e-12, maxit=300, line_search=line_search,
                                      scale_type=scale_type))
    # the search ends at the rounding level of J (|J| ~ 1.7): the projected gradient there is
    # ~1e-7; the minimiser agrees with scipy's L-BFGS-B
    from scipy.optimize import minimize

    ref = minimize(lambda x: fg(x)[0], np.zeros(8), jac=lambda x: fg(x)[1], method="L-BFGS-B",
                   bounds=list(zip(lb, ub)), options={"ftol": 1e-15, "gtol": 1e-12})
    assert res.gnorm < 1e-6, (res.reason, res.gnorm)
    assert np.all(res.x >= lb) and np.all(res.x <= ub)
    assert np.linalg.norm(res.x - ref.x) < 1e-6 * np.linalg.norm(ref.x)


def test_diagonal_scaling_learns_a_diagonal_hessian():
    from glia_gb300.inversion import InitialScaling

    d = np.array([1.0, 10.0, 100.0, 1000.0])
    h0 = InitialScaling("diagonal", 4, 5)
    rng = np.random.default_rng(2)
    ratios = []
    for k in range(400):
        s = rng.standard_normal(4)
        h0.update(s, d * s)
        if k in (0, 399):
            ratios.append(np.max(h0.B / d) / np.min(h0.B / d))
    # from the scalar start (condition ~ 1000 against d) to within a few percent of d
    assert ratios[0] > 100 and ratios[1] < 1.1
    q = np.ones(4)
    assert np.allclose(h0.apply(q, 1.0), 1.0 / h0.B)
