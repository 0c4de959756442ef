"""The named workloads against the FP64 oracle, at their full sizes (needs a GPU).

- 64^3 plain forward (FP64): one Gaussian (sigma = 2pi/64, amplitude 1) at the grid centre,
  kappa = 0.05, k = kappa (wm + 0.2 gm), rho = 10, dt = 0.01, nt = 100, PCG rtol 1e-6 with the
  spectral preconditioner, Strang splitting. c(1) rel-L2 <= 1e-5 (FP64) / 1e-4 (mixed) and equal
  PCG iteration counts per solve (FP64).
- 256^3 forward + adjoint gradient (nt = 100, 512 Gaussians, checkpoints every 10 steps): J and
  the 514-entry gradient against the oracle's full evaluation stored in
  tests/golden/workload256.json (made by tests/golden/make_config1.py), mixed <= 1e-4 and
  FP64 <= 1e-6 relative.
"""
import os

import numpy as np
import pytest

from glia_gb300 import _abi
from glia_gb300 import synthetic as syn
from tests.gpu_common import FP64, MIXED, STATE_TOL, gpu, orc
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _forward64(ctx, nt):
    n = 64
    wl = syn.GradientWorkload(n=n, nt=nt, n_gauss=1, rho=10.0, kappa=0.05, k_gm_wm=0.2)
    tissue = wl.tissue()
    ctx.set_time(wl.dt, nt, 2)
    ctx.set_tissue(*tissue.flat())
    ctx.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    ctx.set_phi(np.array([[np.pi, np.pi, np.pi]]), wl.sigma, 1.0)
    ctx.set_opt(np=1, nk=1, nr=1)
    ctx.set_history(_abi.GLIA_HISTORY_FULL, 0, 0)
    return ctx.phi_apply(np.array([1.0]))


@pytest.fixture(scope="module")
def oracle64():
    o = orc(64)
    c0 = _forward64(o, 100)
    c1 = o.solve_state(c0)
    st = o.stats()
    states = {i: o.get_state(i) for i in (1, 50)}
    # step by step: per-solve PCG counts (the second solve's is last_ksp_itr)
    o2 = orc(64)
    c = _forward64(o2, 1)
    per_solve = []
    for _ in range(100):
        before = o2.stats()["diff_ksp_itr_state"]
        c = o2.solve_state(c)
        s = o2.stats()
        per_solve += [s["diff_ksp_itr_state"] - before - s["last_ksp_itr"], s["last_ksp_itr"]]
    return c0, c1, st, states, per_solve, c


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_forward_64_matches_the_oracle(oracle64, prec):
    c0o, c1o, sto, states, per_solve, c_steps = oracle64
    assert np.linalg.norm(c0o) > 0 and np.linalg.norm(c1o) > 0
    g = gpu(64, prec)
    c0 = _forward64(g, 100)
    assert rel_l2(c0, c0o) < (1e-12 if prec == FP64 else 2e-6)
    c1 = g.solve_state(c0)
    assert rel_l2(c1, c1o) <= STATE_TOL[prec]
    for i, s in states.items():
        assert rel_l2(g.get_state(i), s) <= STATE_TOL[prec]
    if prec == FP64:
        st = g.stats()
        assert st["diff_ksp_itr_state"] == sto["diff_ksp_itr_state"]
        assert st["max_ksp_itr"] == sto["max_ksp_itr"]
        g2 = gpu(64, prec)
        c = _forward64(g2, 1)
        got = []
        for _ in range(100):
            before = g2.stats()["diff_ksp_itr_state"]
            c = g2.solve_state(c)
            s = g2.stats()
            got += [s["diff_ksp_itr_state"] - before - s["last_ksp_itr"], s["last_ksp_itr"]]
        assert got == per_solve
        assert rel_l2(c, c_steps) <= STATE_TOL[prec]


def _workload256(prec, every, engine=_abi.GLIA_ENGINE_FUSED):
    from tests.golden.make_config1 import load, load_data

    want = load(256)
    d = load_data(256)
    wl = syn.GradientWorkload(n=256, nt=want["nt"])
    tissue = wl.tissue()
    centers = wl.centers(tissue)
    g = gpu(256, prec, engine)
    syn.setup_context(g, wl, tissue, centers,
                      _abi.GLIA_HISTORY_CHECKPOINT if every else _abi.GLIA_HISTORY_FULL, every)
    g.set_obs_filter(np.ones(256 ** 3))
    assert np.array_equal(wl.x_eval(), np.array(want["x"]))
    return g, want, d


def _grad_errors(dJ, want_dJ, np_=512):
    w = np.array(want_dJ)
    return (np.linalg.norm(dJ - w) / np.linalg.norm(w),
            np.linalg.norm(dJ[:np_] - w[:np_]) / np.linalg.norm(w[:np_]),
            abs(dJ[np_] - w[np_]) / abs(w[np_]), abs(dJ[np_ + 1] - w[np_ + 1]) / abs(w[np_ + 1]))


@pytest.mark.parametrize("prec,tol", [(MIXED, 1e-4), (FP64, 1e-6)])
def test_gradient_256_matches_the_oracle_fixture(prec, tol):
    if not os.path.exists(os.path.join(GOLDEN, "workload256.json")):
        pytest.fail("tests/golden/workload256.json is missing (tests/golden/make_config1.py)")
    g, want, d = _workload256(prec, 10)
    J, dJ = g.eval_objective_and_gradient(np.array(want["x"]), d)
    assert abs(J - want["J"]) <= tol * abs(want["J"])
    errs = _grad_errors(dJ, want["dJ"])
    assert max(errs) <= tol, errs
