"""TumorParameters::time_history_off_ (GLIA_HISTORY_OFF): forward-only runs that keep no states.
The state equals the full-history state, the objective is unchanged, nothing is allocated for the
history, and the adjoint, gradient and Hessian report a state error instead of sweeping back over
a history that does not exist."""
import numpy as np
import pytest

from glia_gb300 import _abi


def _run(ctx_factory, mode, n=32, nt=5):
    from tests.gpu_common import configure, observation, small_problem

    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    ctx = ctx_factory(n)
    configure(ctx, wl, tissue, centers, mode, 0)
    ctx.set_obs_filter(np.ones(n ** 3))
    x = np.concatenate([np.linspace(0.2, 0.9, len(centers)), [wl.kappa, wl.rho]])
    d1 = observation(wl, tissue, centers)
    c1 = ctx.solve_state(ctx.phi_apply(x[:-2]))
    J = ctx.eval_objective(x, d1)
    return ctx, x, d1, c1, J


def _orc(n):
    from oracle import oracle

    return oracle.context(n)


def test_oracle_history_off_forward_and_refusals():
    full = _run(_orc, _abi.GLIA_HISTORY_FULL)
    off = _run(_orc, _abi.GLIA_HISTORY_OFF)
    assert np.array_equal(off[3], full[3]) and off[4] == full[4]
    ctx, x, d1 = off[0], off[1], off[2]
    with pytest.raises(RuntimeError):
        ctx.eval_objective_and_gradient(x, d1)
    with pytest.raises(RuntimeError):
        ctx.solve_adjoint(np.zeros(32 ** 3))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [_abi.GLIA_FP64, _abi.GLIA_MIXED])
def test_gpu_history_off(prec):
    from tests.gpu_common import gpu

    full = _run(lambda m: gpu(m, prec), _abi.GLIA_HISTORY_FULL)
    off = _run(lambda m: gpu(m, prec), _abi.GLIA_HISTORY_OFF)
    assert np.array_equal(off[3], full[3]) and off[4] == full[4]
    assert off[0].device_bytes() < full[0].device_bytes()
    ctx, x, d1 = off[0], off[1], off[2]
    with pytest.raises(RuntimeError):
        ctx.eval_objective_and_gradient(x, d1)
    with pytest.raises(RuntimeError):
        ctx.hessian_matvec(np.ones(len(x)))
