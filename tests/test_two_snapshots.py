"""Two-snapshot objective (TumorParameters::two_time_points_, Data::dt0): J gains
h^3/2 ||O0 c(0) - d0||^2 and the p gradient h^3 Phi^T O0^T (O0 c(0) - d0)
(src/grad/DerivativeOperatorsRD.cpp:29-33, 114-120, 148-152, 189-196); the Hessian is refused
(:234). CPU tests on the FP64 oracle: the added term, the gradient against central differences,
the Hessian error, switching back; the GPU test compares the CUDA library with the oracle."""
import numpy as np
import pytest

from glia_gb300 import _abi
from tests.helpers import rel_l2


def _setup(ctx_factory, n=32, nt=4):
    from tests.gpu_common import configure, observation, small_problem

    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    ctx = ctx_factory(n)
    configure(ctx, wl, tissue, centers)
    ctx.set_obs_filter(np.ones(n ** 3))
    ctx.set_opt(all_gradients=0, diffusivity_inversion=0, flag_reaction_inv=0)
    x = np.concatenate([np.linspace(0.2, 0.9, len(centers)), [wl.kappa, wl.rho]])
    d1 = observation(wl, tissue, centers)
    rng = np.random.default_rng(11)
    d0 = 0.3 * rng.random(n ** 3) * (tissue.wm.reshape(-1) > 0.5)
    return ctx, wl, x, d1, d0


def _orc(n):
    from oracle import oracle

    return oracle.context(n)


def test_oracle_two_snapshot_objective_adds_the_t0_mismatch():
    ctx, wl, x, d1, d0 = _setup(_orc)
    n, np_ = wl.n, len(x) - 2
    J1 = ctx.eval_objective(x, d1)
    O0 = (d0 > 0.1).astype(np.float64)
    ctx.set_obs_filter0(O0)
    ctx.set_data0(d0)
    J2 = ctx.eval_objective(x, d1)
    c0 = ctx.phi_apply(x[:np_])
    h3 = (2 * np.pi / n) ** 3
    assert abs((J2 - J1) - 0.5 * h3 * np.sum((O0 * c0 - d0) ** 2)) <= 1e-12 * J2
    with pytest.raises(RuntimeError):  # the reference has no two-snapshot Hessian
        ctx.hessian_matvec(np.ones(len(x)))
    ctx.set_data0(None)
    assert ctx.eval_objective(x, d1) == J1


def test_oracle_two_snapshot_gradient_matches_central_differences():
    ctx, wl, x, d1, d0 = _setup(_orc)
    np_ = len(x) - 2
    ctx.set_pcg(1e-11, 5000)
    ctx.set_obs_threshold0(d0, 0.1)
    ctx.set_data0(d0)
    _, g = ctx.eval_objective_and_gradient(x, d1)
    rng = np.random.default_rng(5)
    for _ in range(2):
        u = np.zeros_like(x)
        u[:np_] = rng.standard_normal(np_)
        u /= np.linalg.norm(u)
        h = 1e-3
        fd = (ctx.eval_objective(x + h * u, d1) - ctx.eval_objective(x - h * u, d1)) / (2 * h)
        assert abs(fd - g @ u) <= 1e-4 * abs(fd), (fd, g @ u)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(_abi.GLIA_FP64, 1e-6), (_abi.GLIA_MIXED, 1e-4)])
def test_gpu_two_snapshot_objective_and_gradient(prec, tol):
    """Bars as the one-snapshot parity test: J to 1e-6 (FP64) / 1e-4 (mixed), gradient 1e-4."""
    from tests.gpu_common import gpu

    out = []
    for factory in (_orc, lambda m: gpu(m, prec)):
        ctx, wl, x, d1, d0 = _setup(factory)
        ctx.set_obs_threshold0(d0, 0.1)
        ctx.set_data0(d0)
        out.append(ctx.eval_objective_and_gradient(x, d1))
        with pytest.raises(RuntimeError):
            ctx.hessian_matvec(np.ones(len(x)))
    (Jo, go), (Jg, gg) = out
    assert abs(Jg - Jo) <= tol * abs(Jo)
    assert rel_l2(gg, go) < 1e-4
