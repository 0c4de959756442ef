"""The bounded L-BFGS inversion (glia_gb300/inversion.py, TAO BLMVM with the More-Thuente line
search and the diagonal initial scaling, the reference's defaults) driving the CUDA library: a
32^3 reconstruction reaches the solution of the same run on the FP64 oracle to 1e-3."""
import numpy as np
import pytest

from glia_gb300.inversion import LbfgsSettings, invert, reference_bounds
from tests.gpu_common import FP64, MIXED, configure, gpu, orc, small_problem

pytestmark = pytest.mark.gpu


def _reconstruct(ctx, settings):
    n, nt = 32, 3
    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    configure(ctx, wl, tissue, centers)
    ctx.set_obs_filter(np.ones(n ** 3))
    ctx.set_pcg(1e-8, 5000, 1, wl.dt)
    x_true = np.concatenate([[0.0, 0.9, 0.0, 0.0, 0.6, 0.0, 0.0, 0.0], [wl.kappa, wl.rho]])
    ctx.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    d = ctx.solve_state(ctx.phi_apply(x_true[:8]))
    lb, ub = reference_bounds(8)
    x0 = np.concatenate([np.zeros(8), [0.7 * wl.kappa, 0.8 * wl.rho]])
    return invert(ctx, d, x0, lb, ub, settings), x_true


@pytest.mark.parametrize("line_search,scale_type", [("mt", "diagonal"), ("armijo", "scalar")])
def test_gpu_reconstruction_reaches_the_oracle_solution(line_search, scale_type):
    s = LbfgsSettings(maxit=25, line_search=line_search, scale_type=scale_type)
    ro, x_true = _reconstruct(orc(32), s)
    rg, _ = _reconstruct(gpu(32, FP64), s)
    assert rg.reason == ro.reason
    assert np.linalg.norm(rg.x - ro.x) <= 1e-3 * np.linalg.norm(ro.x)
    assert abs(rg.J - ro.J) <= 1e-3 * abs(ro.J) + 1e-12
    # and the reconstruction itself recovers the generating coefficients
    assert np.linalg.norm(rg.x[:8] - x_true[:8]) < 0.1 * np.linalg.norm(x_true[:8])


def test_mixed_reconstruction_converges_to_the_same_coefficients():
    s = LbfgsSettings(maxit=25)
    ro, x_true = _reconstruct(orc(32), s)
    rm, _ = _reconstruct(gpu(32, MIXED), s)
    assert rm.gnorm < 1e-2 * rm.gnorm0
    assert np.linalg.norm(rm.x[:8] - ro.x[:8]) <= 1e-2 * np.linalg.norm(ro.x[:8])
