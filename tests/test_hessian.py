"""Gauss-Newton Hessian matvec (DerivativeOperatorsRD::evaluateHessian: the p block, and the p and
kappa blocks with diffusivity inversion) and the linearised solves it is made of (solveState(1),
solveState(2), solveAdjoint(2)).

CPU tests run on the FP64 oracle: linearity, the finite-difference derivative of the gradient at
a zero residual, the call-order error, solveState(2) against a kappa difference of the forward,
and the reference's t = 1 term of the kappa rows (p_[nt] left by the last gradient's adjoint).
GPU tests compare the CUDA library with the oracle in every engine / precision and check
checkpointed == full history."""
import numpy as np
import pytest

from glia_gb300 import _abi
from tests.helpers import rel_l2


def _problem(ctx_factory, n=32, nt=4, n_gauss=8, history=_abi.GLIA_HISTORY_FULL, every=2,
             diffusivity=0):
    from tests.gpu_common import configure, small_problem

    wl, tissue, centers = small_problem(n, nt, n_gauss=n_gauss)
    ctx = ctx_factory(n)
    configure(ctx, wl, tissue, centers, history, every)
    ctx.set_opt(diffusivity_inversion=diffusivity, all_gradients=0, flag_reaction_inv=0)
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


def _grad3(f, n):
    """Spectral gradient with the Nyquist wave numbers set to 0 (computeGradient)."""
    F = np.fft.rfftn(f.reshape(n, n, n))
    k = np.fft.fftfreq(n, 1.0 / n)
    k[n // 2] = 0
    kz = np.fft.rfftfreq(n, 1.0 / n)
    kz[-1] = 0
    K = np.meshgrid(k, k, kz, indexing="ij")
    return [np.fft.irfftn(1j * Kd * F, s=(n, n, n), axes=(0, 1, 2)).reshape(-1) for Kd in K]


def test_oracle_incremental_forward_in_kappa_matches_differences():
    """solveState(2) from c~0 = 0 with k~ = wm + r gm against (c(1; kappa + e) -
    c(1; kappa - e)) / 2e: equal up to the O(dt) of the reference's linearisation (logistic step
    at c_i, diffusion sources from averaged states)."""
    n = 32
    ctx, wl, x, _ = _problem(_orc, n, diffusivity=1)
    ctx.set_pcg(1e-10, 5000, 1, wl.dt)
    np_ = len(x) - 2
    c0 = ctx.phi_apply(x[:np_])
    ctx.solve_state(c0)
    with pytest.raises(RuntimeError):  # no secondary coefficients yet
        ctx.solve_state(np.zeros(n ** 3), linearized=2)
    ctx.set_secondary_coefficients(1.0)
    ct = ctx.solve_state(np.zeros(n ** 3), linearized=2)
    eps, out = 1e-4, []
    for sgn in (1, -1):
        ctx.set_coefficients(k=wl.kappa + sgn * eps, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
        out.append(ctx.solve_state(c0))
    assert rel_l2(ct, (out[0] - out[1]) / (2 * eps)) < 2e-3


def test_oracle_diffusivity_hessian_against_gradient_differences():
    """With diffusivity inversion at a zero residual: linear in x; the p rows are the derivative
    of the p gradient; the kappa row is the derivative of the kappa gradient less the t = 1 term
    0.5 dt h^3 <wm + r gm, grad c(1) . grad a~(1)>, which the reference replaces by p_[nt] (here
    the zero final condition of the gradient's adjoint). Rho rows are 0."""
    n = 32
    ctx, wl, x, rng = _problem(_orc, n, diffusivity=1)
    ctx.set_pcg(1e-10, 5000, 1, wl.dt)
    np_ = len(x) - 2
    d = ctx.solve_state(ctx.phi_apply(x[:np_]))
    J, _ = ctx.eval_objective_and_gradient(x, d)
    assert J < 1e-12
    u = np.concatenate([rng.standard_normal(np_), [0.01, 0.0]])
    v = np.concatenate([rng.standard_normal(np_), [-0.02, 0.0]])
    Hu, Hv = ctx.hessian_matvec(u), ctx.hessian_matvec(v)
    assert rel_l2(ctx.hessian_matvec(2.0 * u - 0.5 * v), 2.0 * Hu - 0.5 * Hv) < 1e-8
    assert Hu[np_ + 1] == 0.0
    eps = 1e-4
    fd = (ctx.eval_gradient(x + eps * u, d) - ctx.eval_gradient(x - eps * u, d)) / (2 * eps)
    assert rel_l2(Hu[:np_], fd[:np_]) < 2e-3
    # the t = 1 term from the incremental state of the whole direction
    ctx.eval_objective_and_gradient(x, d)
    ct = ctx.solve_state(ctx.phi_apply(u[:np_]), linearized=1)
    ctx.set_secondary_coefficients(u[np_])
    ct = ct + ctx.solve_state(np.zeros(n ** 3), linearized=2)
    gc, ga = _grad3(ctx.get_state(wl.nt), n), _grad3(-ct, n)
    t1 = 0.5 * wl.dt * (gc[0] * ga[0] + gc[1] * ga[1] + gc[2] * ga[2])
    _, tissue, _ = _tissue(n, wl.nt)
    m = tissue.wm.reshape(-1) + wl.k_gm_wm * tissue.gm.reshape(-1)
    h3 = (2 * np.pi / n) ** 3
    assert abs(Hu[np_] + h3 * (m @ t1) - fd[np_]) < 2e-3 * abs(fd[np_])
    assert abs(Hu[np_] - fd[np_]) > 0.05 * abs(fd[np_])  # the term is not negligible


def test_oracle_diffusivity_hessian_reads_the_last_gradients_final_condition():
    """The kappa rows take p_[nt] from the last linearized = 1 adjoint: two gradients at the same
    x with different data leave the same history but different p_[nt]; the p rows agree, the
    kappa row does not."""
    ctx, wl, x, rng = _problem(_orc, diffusivity=1)
    np_ = len(x) - 2
    d = ctx.solve_state(ctx.phi_apply(0.8 * x[:np_]))
    u = np.concatenate([rng.standard_normal(np_), [0.01, 0.0]])
    ctx.eval_objective_and_gradient(x, d)
    H1 = ctx.hessian_matvec(u)
    ctx.eval_objective_and_gradient(x, 0.5 * d)
    H2 = ctx.hessian_matvec(u)
    assert rel_l2(H2[:np_], H1[:np_]) < 1e-12
    assert abs(H2[np_] - H1[np_]) > 1e-6 * abs(H1[np_])


def _tissue(n, nt):
    from tests.gpu_common import small_problem

    return small_problem(n, nt, n_gauss=8)


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


@pytest.mark.gpu
@pytest.mark.parametrize("precision,engine,history,tol,n", [
    (_abi.GLIA_FP64, _abi.GLIA_ENGINE_FUSED, _abi.GLIA_HISTORY_FULL, 1e-9, 32),
    (_abi.GLIA_FP64, _abi.GLIA_ENGINE_FUSED, _abi.GLIA_HISTORY_CHECKPOINT, 1e-9, 32),
    (_abi.GLIA_FP64, _abi.GLIA_ENGINE_REFERENCE, _abi.GLIA_HISTORY_FULL, 1e-9, 32),
    (_abi.GLIA_MIXED, _abi.GLIA_ENGINE_FUSED, _abi.GLIA_HISTORY_FULL, 1e-4, 32),
    (_abi.GLIA_MIXED, _abi.GLIA_ENGINE_FUSED, _abi.GLIA_HISTORY_CHECKPOINT, 1e-4, 32),
    # 64^3 FP32: the own x / y / z transform kernels, whose z pass reads k~ for the D~ apply
    (_abi.GLIA_MIXED, _abi.GLIA_ENGINE_FUSED, _abi.GLIA_HISTORY_CHECKPOINT, 1e-4, 64),
])
def test_gpu_diffusivity_hessian_matches_oracle(precision, engine, history, tol, n):
    """Hessian with diffusivity inversion (p and kappa blocks, the t = 1 term from p_[nt]) and
    solveState(2) against the oracle, at a nonzero residual so that p_[nt] is not 0."""
    from tests.gpu_common import gpu

    octx, wl, x, rng = _problem(_orc, n, nt=6, diffusivity=1)
    gctx, _, _, _ = _problem(lambda m: gpu(m, precision, engine), n, nt=6, history=history,
                             every=4, diffusivity=1)
    np_ = len(x) - 2
    if precision == _abi.GLIA_FP64:
        # a tight PCG tolerance, so that a convergence test decided one iteration apart by
        # rounding (GPU: spectral-space PCG) cannot show at the rtol level in the comparison
        for ctx in (octx, gctx):
            ctx.set_pcg(1e-10, 5000, 1, wl.dt)
    d = octx.solve_state(octx.phi_apply(0.8 * x[:np_]))
    u = np.concatenate([rng.standard_normal(np_), [0.01, 0.0]])
    for ctx in (octx, gctx):
        ctx.eval_objective_and_gradient(x, d)
    Hg, Ho = gctx.hessian_matvec(u), octx.hessian_matvec(u)
    assert rel_l2(Hg, Ho) < tol
    assert abs(Hg[np_] - Ho[np_]) < tol * abs(Ho[np_])
    for ctx in (octx, gctx):
        ctx.set_secondary_coefficients(0.02)
    z = np.zeros(n ** 3)
    assert rel_l2(gctx.solve_state(z, linearized=2), octx.solve_state(z, linearized=2)) < tol
