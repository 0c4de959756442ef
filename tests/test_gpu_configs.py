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


def steady_pc(ctx, dt):
    """The reference's preconditioner takes the dt of the last diffusion solve at the time it is
    built (DiffusionSolver::precFactor reads the solver's context dt, which solve overwrites;
    src/pde/DiffusionSolver.cpp:140,165 vs :226). Every evaluation after a context's first one
    therefore runs with the Strang half step dt/2; a fresh context's first one uses the full dt.
    At rtol 1e-6 the two preconditioners give PCG iterates that differ by ~1e-5 in J and ~1e-4
    in the gradient. One solve at dt/2 puts a fresh context in the steady state, which is the
    state of the oracle fixture's evaluation (it follows the observation forward) and of the
    bench's timed steps (they follow warm-up evaluations)."""
    ctx.diffusion_solve(np.ones(ctx.N), dt / 2)


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
    steady_pc(g, wl.dt)
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


def _data256(g, wl):
    """The oracle's observation when the fixture exists, else this FP64 path's own forward with
    the perturbed parameters, thresholded at 0.5."""
    if os.path.exists(os.path.join(GOLDEN, "workload256_data.npz")):
        from tests.golden.make_config1 import load_data

        return load_data(256), "oracle fixture"
    g.set_coefficients(k=wl.kappa * 0.8, rho=wl.rho * 1.2, k_gm_wm=wl.k_gm_wm)
    c1 = g.solve_state(g.phi_apply(wl.p_obs()))
    g.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    return (c1 > 0.5).astype(np.float64), "FP64 GPU forward"


@pytest.mark.skipif(os.environ.get("GLIA_SLOW") != "1",
                    reason="opt-in (GLIA_SLOW=1): 16 FP64 objective evaluations at 256^3, ~7 min")
def test_gradient_256_central_differences():
    """DerivativeOperators::checkGradient's protocol (src/grad/DerivativeOperators.cpp:369-450)
    on the 256^3 workload: central differences (h = 1e-3) of J along 8 random unit directions
    (seed 3) against the adjoint gradient taken through the torch.autograd.Function
    (glia_gb300.autograd.rd_objective, the data a CUDA tensor: the device-pointer path), FP64
    fused path, PCG rtol 1e-10 so that the PCG tolerance stays below the difference quotient's
    resolution. The p block is the exact discrete adjoint; kappa and rho are the reference's
    trapezoid quadratures."""
    import json
    import time

    import torch

    from glia_gb300 import autograd as ga

    wl = syn.GradientWorkload(n=256, nt=100)
    tissue = wl.tissue()
    centers = wl.centers(tissue)
    g = gpu(256, FP64)
    syn.setup_context(g, wl, tissue, centers, _abi.GLIA_HISTORY_CHECKPOINT, 10)
    g.set_obs_filter(np.ones(256 ** 3))
    g.set_pcg(1e-10, 5000)
    d1, source = _data256(g, wl)
    steady_pc(g, wl.dt)
    d1_dev = torch.tensor(d1, dtype=torch.float64, device="cuda")
    x = wl.x_eval()
    t0 = time.time()
    xt = torch.tensor(x, requires_grad=True)
    Jt = ga.rd_objective(xt, g, d1_dev)
    Jt.backward()
    J, grad = float(Jt.detach()), xt.grad.numpy().copy()
    rng = np.random.default_rng(3)
    h, np_ = 1e-3, wl.n_gauss
    rows = []
    for _ in range(8):
        d = rng.standard_normal(x.size)
        d /= np.linalg.norm(d)
        Jp = float(ga.rd_objective(torch.tensor(x + h * d), g, d1_dev))
        Jm = float(ga.rd_objective(torch.tensor(x - h * d), g, d1_dev))
        fd = (Jp - Jm) / (2 * h)
        ad = float(grad @ d)
        rows.append({"fd": fd, "adjoint": ad, "rel_err": abs(fd - ad) / abs(fd),
                     "p_part": float(grad[:np_] @ d[:np_]),
                     "kappa_part": float(grad[np_] * d[np_]),
                     "rho_part": float(grad[np_ + 1] * d[np_ + 1])})
    out = {"J": J, "data": source, "h": h, "rtol": 1e-10, "seconds": time.time() - t0,
           "directions": rows, "max_rel_err": max(r["rel_err"] for r in rows)}
    path = os.environ.get("GLIA_FD_OUT")
    if path:
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
    print(json.dumps(out))
    # GB300, FP64, data of this path's own forward: worst direction 3.3e-5 (kappa dominates)
    assert out["max_rel_err"] <= 1e-4


@pytest.mark.skipif(os.environ.get("GLIA_SLOW") != "1",
                    reason="opt-in (GLIA_SLOW=1): one FP64 evaluation at 256^3 with 1000 Gaussians")
def test_gradient_256_1000_gaussians_mixed_vs_fp64():
    """The 256^3 reconstruction's problem (1000 Gaussians at the first in-brain lattice points,
    5 active, rho = 10, kappa = 0.05, nt = 100, checkpoints every 10): the mixed path's gradient
    at the reconstruction's starting point and halfway to the truth against the FP64 path's,
    <= 1e-4 (the workload's gradient bar). J = h^3/2 ||c(1) - d||^2 is a squared distance to the
    data, so its relative error grows as it nears the minimum; it is held to 5e-4.
    GB300: gradient 3.7e-5 / 2.2e-5, J 1.7e-5 / 1.1e-4 (start / halfway)."""
    import json

    from glia_gb300.inversion import reconstruction_256

    wl, tissue, centers, x_true, _ = reconstruction_256()
    ctxs = {}
    for prec in (FP64, MIXED):
        g = gpu(256, prec)
        syn.setup_context(g, wl, tissue, centers, _abi.GLIA_HISTORY_CHECKPOINT, 10)
        g.set_obs_filter(np.ones(256 ** 3))
        ctxs[prec] = g
    gen = ctxs[FP64]
    gen.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    d1 = gen.solve_state(gen.phi_apply(x_true[:-2]))
    steady_pc(ctxs[MIXED], wl.dt)  # the FP64 context's last solve was the forward's dt/2
    npp = len(centers)
    x0 = np.concatenate([0.1 * (x_true[:npp] > 0), [0.5 * wl.kappa, 0.5 * wl.rho]])
    # the reconstruction's start and a point halfway to the truth (at the truth itself J and
    # the gradient vanish up to the solver tolerance, and relative errors lose their meaning)
    half = np.concatenate([0.5 * x_true[:npp], [0.75 * wl.kappa, 0.75 * wl.rho]])
    out = {}
    for name, x in (("start", x0), ("halfway", half)):
        got = {prec: ctxs[prec].eval_objective_and_gradient(x, d1) for prec in (MIXED, FP64)}
        (Jm, gm), (Jd, gd) = got[MIXED], got[FP64]
        out[name] = {"J_rel": abs(Jm - Jd) / abs(Jd),
                     "grad_rel": float(np.linalg.norm(gm - gd) / np.linalg.norm(gd))}
    print(json.dumps(out))
    for v in out.values():
        assert v["grad_rel"] <= 1e-4 and v["J_rel"] <= 5e-4
