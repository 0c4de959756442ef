"""The FP64 CPU oracle against the reference's own known answers and against numpy.

- src/test/pdesolver.cpp:46-48: ||c||_2 == Approx(2.0487) and ksp_itr_ == 5 after 10 CN solves.
- src/test/grad.cpp:74-77: J < 1e-7 at the generating parameters, J > 0 with zero data.
- the oracle's hand-written 3-D R2C/C2R against numpy.fft.
"""
import numpy as np
import pytest

from glia_gb300 import _abi
from oracle import oracle
from tests.helpers import reference_test_field

# Catch2's Approx default: epsilon = 100 * float epsilon, relative to the value
CATCH_EPS = 100 * np.finfo(np.float32).eps


@pytest.mark.parametrize("n", [8, 16, 32])
def test_fft_matches_numpy(n):
    api = oracle.load()
    x = np.random.default_rng(n).standard_normal(n ** 3)
    spec = np.zeros(n * n * (n // 2 + 1) * 2)
    api.fft_r2c(n, x.ctypes.data, spec.ctypes.data)
    ref = np.fft.rfftn(x.reshape(n, n, n))
    got = spec.view(np.complex128).reshape(ref.shape)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    back = np.zeros(n ** 3)
    api.fft_c2r(n, spec.ctypes.data, back.ctypes.data)
    assert np.abs(back / n ** 3 - x).max() < 1e-12


def run_pdesolver(ctx, n=64):
    """src/test/pdesolver.cpp:7-48 step by step."""
    c = reference_test_field(n)
    ctx.set_diffusivity_sinusoidal(1e-2)      # k->setValuesSinusoidal(params, 1E-2)
    ctx.set_time(0.5, 1, 2)                   # DiffusionSolver built with TumorParameters::dt_
    ctx.prec_factor()                         # diff_solver->precFactor()
    its = None
    for _ in range(10):
        its = ctx.diffusion_solve(c, 0.02)
    return c, its


def test_pdesolver_known_answer():
    ctx = oracle.context(64)
    c, its = run_pdesolver(ctx)
    nrm = np.linalg.norm(c)
    assert abs(nrm - 2.0487) <= CATCH_EPS * 2.0487, nrm
    assert its == 5


def test_pdesolver_pin_discriminates_pc_convention():
    # the 5-iteration pin holds only with the reference's PC-dt rule (PC built at dt_ = 0.5)
    ctx = oracle.context(64)
    ctx.set_pcg(1e-6, 5000, _abi.GLIA_PC_DT_MATCHED, 0.0)
    _, its = run_pdesolver(ctx)
    assert its != 5


def test_grad_objective_known_answer():
    """src/test/grad.cpp:7-80 at 64^3, dt = 0.01, nt = 100, sinusoidal tissue."""
    n = 64
    ctx = oracle.context(n)
    ctx.set_time(0.01, 100, 2)
    ctx.set_tissue_sinusoidal()
    ctx.set_coefficients(k=0.01, rho=10.0)
    ctx.set_opt(np=1, nk=1, nr=1, flag_reaction_inv=1, diffusivity_inversion=1, beta=0.0)
    kt = rt = 0.01  # the test sets rho to kappa's value (rt = k_, src/test/grad.cpp:49)
    x = np.array([0.0, kt, rt])
    zeros = np.zeros(n ** 3)
    ctx.set_c0(reference_test_field(n))
    ctx.eval_objective(x, zeros)              # updateReactionAndDiffusion + solveState
    data = ctx.get_state(100)
    j_true = ctx.eval_objective(x, data)
    assert j_true < 1e-7
    j_zero = ctx.eval_objective(x, zeros)
    assert j_zero > 0
