"""CUDA library against the FP64 CPU oracle on the same seeded inputs (needs a GPU).

Every comparison goes through the C-ABI (include/glia_rd.h). Bars: FP64 state rel-L2 <= 1e-5,
mixed (FP32 bulk, FP64 reductions) <= 1e-4, gradients <= 1e-4; PCG iteration counts equal for
FP64.
"""
import numpy as np
import pytest

from glia_gb300 import _abi
from tests.gpu_common import (FP64, FUSED, GRAD_TOL, MIXED, REFERENCE, STATE_TOL, configure,
                              gpu, observation, orc, small_problem)
from tests.helpers import reference_test_field, rel_l2
from tests.test_oracle_pins import CATCH_EPS, run_pdesolver

pytestmark = pytest.mark.gpu

ENGINES = [(FP64, FUSED), (MIXED, FUSED), (FP64, REFERENCE)]


@pytest.mark.parametrize("prec,eng", ENGINES + [(MIXED, REFERENCE)])
def test_pdesolver_known_answer(prec, eng):
    """src/test/pdesolver.cpp:46-48 through glia_diffusion_solve."""
    c, its = run_pdesolver(gpu(64, prec, eng))
    nrm = np.linalg.norm(c)
    tol = CATCH_EPS * 2.0487 if prec == FP64 else 1e-4 * 2.0487
    assert abs(nrm - 2.0487) <= tol, nrm
    assert its == 5


@pytest.mark.parametrize("prec,eng", ENGINES)
def test_apply_d_and_smoother(prec, eng):
    n = 32
    wl, tissue, centers = small_problem(n)
    o, g = orc(n), gpu(n, prec, eng)
    for ctx in (o, g):
        configure(ctx, wl, tissue, centers)
    f = reference_test_field(n) + 0.1 * tissue.wm.reshape(-1)
    tol = 1e-11 if prec == FP64 else 2e-5
    assert rel_l2(g.apply_d(f), o.apply_d(f)) < tol
    s = 2 * np.pi / n
    assert rel_l2(g.smooth(f, s), o.smooth(f, s)) < tol


@pytest.mark.parametrize("prec", [FP64, MIXED])
@pytest.mark.parametrize("phi_store", [0, 1])
def test_phi_apply_and_transpose(prec, phi_store):
    n = 32
    wl, tissue, centers = small_problem(n, n_gauss=8)
    o, g = orc(n), gpu(n, prec)
    for ctx in (o, g):
        configure(ctx, wl, tissue, centers)
        ctx.set_opt(phi_store=phi_store)
    p = np.linspace(0.0, 1.0, len(centers))
    p[1] = 0.0
    tol = 1e-12 if prec == FP64 else 2e-6
    assert rel_l2(g.phi_apply(p), o.phi_apply(p)) < tol
    v = reference_test_field(n) + tissue.gm.reshape(-1)
    assert rel_l2(g.phi_apply_transpose(v, len(p)), o.phi_apply_transpose(v, len(p))) < tol


@pytest.mark.parametrize("prec,eng", ENGINES)
def test_solve_state_and_adjoint(prec, eng):
    n, nt = 32, 6
    wl, tissue, centers = small_problem(n, nt)
    o, g = orc(n), gpu(n, prec, eng)
    for ctx in (o, g):
        configure(ctx, wl, tissue, centers)
        ctx.set_history(_abi.GLIA_HISTORY_FULL, 0, 0)
    p = np.zeros(len(centers))
    p[:3] = [1.0, 0.5, 0.25]
    c0 = o.phi_apply(p)
    c1o, c1g = o.solve_state(c0), g.solve_state(c0)
    assert rel_l2(c1g, c1o) < STATE_TOL[prec]
    so, sg = o.stats(), g.stats()
    if prec == FP64:
        assert sg["diff_ksp_itr_state"] == so["diff_ksp_itr_state"]
    for i in (1, nt // 2):
        assert rel_l2(g.get_state(i), o.get_state(i)) < STATE_TOL[prec]
    pt = -(c1o - 0.5 * c1o.max())
    a0o, a0g = o.solve_adjoint(pt), g.solve_adjoint(pt)
    assert rel_l2(a0g, a0o) < STATE_TOL[prec]


@pytest.mark.parametrize("prec,eng", ENGINES)
def test_objective_and_gradient(prec, eng):
    n, nt = 32, 6
    wl, tissue, centers = small_problem(n, nt)
    d1 = observation(wl, tissue, centers)
    o, g = orc(n), gpu(n, prec, eng)
    for ctx in (o, g):
        configure(ctx, wl, tissue, centers)
        ctx.set_obs_filter(np.ones(n ** 3))
    x = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    Jo, gro = o.eval_objective_and_gradient(x, d1)
    Jg, grg = g.eval_objective_and_gradient(x, d1)
    assert abs(Jg - Jo) <= 1e-6 * abs(Jo) if prec == FP64 else abs(Jg - Jo) <= 1e-4 * abs(Jo)
    assert rel_l2(grg, gro) < GRAD_TOL
    # each block of the gradient on its own
    np_ = len(centers)
    assert rel_l2(grg[:np_], gro[:np_]) < GRAD_TOL
    assert abs(grg[np_] - gro[np_]) <= GRAD_TOL * abs(gro[np_])
    assert abs(grg[np_ + 1] - gro[np_ + 1]) <= GRAD_TOL * abs(gro[np_ + 1])


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_checkpointed_gradient_equals_full_history(prec):
    n, nt = 32, 10
    wl, tissue, centers = small_problem(n, nt)
    d1 = observation(wl, tissue, centers)
    x = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    out = []
    for hist, every in ((_abi.GLIA_HISTORY_FULL, 0), (_abi.GLIA_HISTORY_CHECKPOINT, 3),
                        (_abi.GLIA_HISTORY_CHECKPOINT, 10)):
        g = gpu(n, prec)
        configure(g, wl, tissue, centers, hist, every)
        g.set_obs_filter(np.ones(n ** 3))
        out.append(g.eval_objective_and_gradient(x, d1))
    for J, gr in out[1:]:
        assert J == out[0][0]
        assert rel_l2(gr, out[0][1]) < 1e-12


def test_grad_objective_known_answer_gpu():
    """src/test/grad.cpp:7-80 on the CUDA library (FP64, 64^3, nt = 100)."""
    n = 64
    g = gpu(n, FP64)
    g.set_time(0.01, 100, 2)
    g.set_tissue_sinusoidal()
    g.set_coefficients(k=0.01, rho=10.0)
    g.set_opt(np=1, nk=1, nr=1, flag_reaction_inv=1, diffusivity_inversion=1, beta=0.0)
    x = np.array([0.0, 0.01, 0.01])
    zeros = np.zeros(n ** 3)
    g.set_c0(reference_test_field(n))
    g.eval_objective(x, zeros)
    data = g.get_state(100)
    assert g.eval_objective(x, data) < 1e-7
    assert g.eval_objective(x, zeros) > 0


def test_gradient_matches_central_differences():
    """Adjoint p-gradient vs central finite differences (h = 1e-3) on random directions."""
    n, nt = 32, 6
    wl, tissue, centers = small_problem(n, nt)
    d1 = observation(wl, tissue, centers)
    g = gpu(n, FP64)
    configure(g, wl, tissue, centers)
    g.set_obs_filter(np.ones(n ** 3))
    g.set_opt(all_gradients=0, diffusivity_inversion=0)  # p only: the exact discrete adjoint
    g.set_pcg(1e-11, 5000)  # converged solves, so J is smooth in x
    x = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    _, gr = g.eval_objective_and_gradient(x, d1)
    rng = np.random.default_rng(3)
    for _ in range(3):
        d = np.zeros_like(x)
        d[: len(centers)] = rng.standard_normal(len(centers))
        d /= np.linalg.norm(d)
        h = 1e-3
        fd = (g.eval_objective(x + h * d, d1) - g.eval_objective(x - h * d, d1)) / (2 * h)
        assert abs(fd - gr @ d) <= 1e-4 * max(abs(fd), 1e-12), (fd, gr @ d)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_graph_loop_equals_host_loop(prec):
    """The PCG loop as a CUDA graph with a device-side WHILE node gives the same bits as the
    host-driven loop (used while per-kernel timing is on)."""
    n, nt = 32, 4
    wl, tissue, centers = small_problem(n, nt)
    d1 = observation(wl, tissue, centers)
    x = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    out = []
    for timing in (False, True):
        g = gpu(n, prec)
        configure(g, wl, tissue, centers)
        g.set_obs_filter(np.ones(n ** 3))
        g.set_timing(timing)
        out.append(g.eval_objective_and_gradient(x, d1) + (g.stats(),))
    (J0, g0, s0), (J1, g1, s1) = out
    assert J0 == J1 and np.array_equal(g0, g1)
    assert s0["diff_ksp_itr_state"] == s1["diff_ksp_itr_state"]
    assert s0["diff_ksp_itr_adj"] == s1["diff_ksp_itr_adj"]


@pytest.mark.parametrize("n", [64, 128, 256])
def test_fused_zpass_matches_cufft_3d_path(n, monkeypatch):
    """FP32 D apply with the fused z pass (k_zpass_mulk between 2-D cuFFT passes) against the
    three-dimensional cuFFT transforms around k_mul_k3 (GLIA_XPASS=0)."""
    wl, tissue, centers = small_problem(n, 2, n_gauss=8)
    f = reference_test_field(n) + 0.1 * tissue.wm.reshape(-1)
    out = []
    for zpass, xpass in (("1", "own"), ("0", "0")):
        monkeypatch.setenv("GLIA_ZPASS", zpass)
        monkeypatch.setenv("GLIA_XPASS", xpass)  # "0": batched 3-D cuFFT
        g = gpu(n, MIXED)
        configure(g, wl, tissue, centers)
        out.append((g.apply_d(f), g.solve_state(g.phi_apply(np.linspace(0.2, 1, 8)))))
    assert rel_l2(out[0][0], out[1][0]) < 2e-6
    assert rel_l2(out[0][1], out[1][1]) < 1e-5


@pytest.mark.parametrize("path", ["own", "own_tma", "2d", "zpass"])
@pytest.mark.parametrize("n", [64, 128])
def test_transform_paths_against_oracle(n, path, monkeypatch):
    """D apply, state and gradient of the FP32 transform paths against the FP64 oracle: the
    default own x / y / z kernels, the x pass around 2-D cuFFT, the fused z pass."""
    if path == "zpass":
        monkeypatch.setenv("GLIA_ZPASS", "1")
    elif path == "own_tma":  # y-forward pass staged by TMA tensor copies
        monkeypatch.setenv("GLIA_TMA", "1")
    elif path == "2d":
        monkeypatch.setenv("GLIA_XPASS", "2d")
    nt = 4
    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    o, g = orc(n), gpu(n, MIXED)
    for ctx in (o, g):
        configure(ctx, wl, tissue, centers)
    f = reference_test_field(n) + 0.1 * tissue.wm.reshape(-1)
    assert rel_l2(g.apply_d(f), o.apply_d(f)) < 2e-5
    p = np.linspace(0.2, 1.0, len(centers))
    c0 = o.phi_apply(p)
    assert rel_l2(g.solve_state(c0), o.solve_state(c0)) < STATE_TOL[MIXED]
    d1 = observation(wl, tissue, centers)
    for ctx in (o, g):
        ctx.set_obs_filter(np.ones(n ** 3))
    x = np.concatenate([p, [wl.kappa, wl.rho]])
    _, gro = o.eval_objective_and_gradient(x, d1)
    _, grg = g.eval_objective_and_gradient(x, d1)
    assert rel_l2(grg, gro) < GRAD_TOL


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_full_size_d_apply_and_cn_solve(prec):
    """256^3, the size of the gradient-evaluation workload: D apply and one Crank-Nicolson
    diffusion solve against the oracle, equal PCG iteration counts (FP64), and two properties of
    the operator that hold at every size: D u sums to zero (the divergence has no mean) and D is
    symmetric, <D u, v> = <u, D v>; the solve conserves mass."""
    n = 256
    wl, tissue, centers = small_problem(n, 2, n_gauss=1)
    o, g = orc(n), gpu(n, prec)
    for ctx in (o, g):
        configure(ctx, wl, tissue, centers)
    f = reference_test_field(n) + 0.1 * tissue.wm.reshape(-1)
    v = reference_test_field(n)[::-1].copy() + tissue.gm.reshape(-1)
    tol = 1e-11 if prec == FP64 else 2e-5
    df = g.apply_d(f)
    assert rel_l2(df, o.apply_d(f)) < tol
    dv = g.apply_d(v)
    assert abs(df.sum()) <= tol * np.abs(df).sum()
    assert abs(np.dot(df, v) - np.dot(f, dv)) <= tol * np.linalg.norm(df) * np.linalg.norm(v)
    cg, co = f.copy(), f.copy()
    its_g = g.diffusion_solve(cg, wl.dt)
    its_o = o.diffusion_solve(co, wl.dt)
    assert rel_l2(cg, co) < STATE_TOL[prec]
    if prec == FP64:
        assert its_g == its_o
    assert abs(cg.sum() - f.sum()) <= (1e-12 if prec == FP64 else 1e-5) * np.abs(f).sum()


def test_repeated_adjoint_after_one_state_solve_checkpointed():
    """Two adjoint sweeps after one state solve (checkpointed history) give the same result."""
    n, nt = 32, 7
    wl, tissue, centers = small_problem(n, nt)
    g = gpu(n, MIXED)
    configure(g, wl, tissue, centers, _abi.GLIA_HISTORY_CHECKPOINT, 3)
    c1 = g.solve_state(g.phi_apply(np.linspace(0.2, 1.0, len(centers))))
    pt = -(c1 - 0.5 * c1.max())
    a = g.solve_adjoint(pt)
    b = g.solve_adjoint(pt)
    assert np.array_equal(a, b)
    f = gpu(n, MIXED)
    configure(f, wl, tissue, centers)
    f.solve_state(f.phi_apply(np.linspace(0.2, 1.0, len(centers))))
    assert rel_l2(a, f.solve_adjoint(pt)) < 1e-12


@pytest.mark.parametrize("path", ["own", "own_tma", "own_evenodd", "own_yinv_cpasync", "2d"])
@pytest.mark.parametrize("n", [64, 128, 256])
def test_transform_paths_match_cufft_3d(n, path, monkeypatch):
    """FP32 D apply, state solve and gradient through the library's own x / y / z transform
    kernels ("own": k_xinv, k_yinv_bulk, k_zpass2, k_yfwd, k_xfwd; "own_evenodd": the even/odd
    z pass k_zpass; "own_yinv_cpasync": k_yinv) and through the x pass around batched 2-D cuFFT
    ("2d"), against the batched 3-D cuFFT path."""
    nt = 3
    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    d1 = observation(wl, tissue, centers)
    f = reference_test_field(n) + 0.1 * tissue.wm.reshape(-1)
    x = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    out = []
    if path == "own_tma":  # y-forward pass staged by TMA tensor copies
        monkeypatch.setenv("GLIA_TMA", "1")
    if path == "own_evenodd":
        monkeypatch.setenv("GLIA_ZPASS2", "0")
    if path == "own_yinv_cpasync":  # y-inverse rows staged by per-thread cp.async
        monkeypatch.setenv("GLIA_YINV_BULK", "0")
    for on in (path, "0"):
        monkeypatch.setenv("GLIA_XPASS", on)
        g = gpu(n, MIXED)
        configure(g, wl, tissue, centers)
        g.set_obs_filter(np.ones(n ** 3))
        c0 = g.phi_apply(np.linspace(0.2, 1.0, len(centers)))
        out.append((g.apply_d(f), g.solve_state(c0), g.eval_objective_and_gradient(x, d1)))
    assert rel_l2(out[0][0], out[1][0]) < 2e-6
    assert rel_l2(out[0][1], out[1][1]) < 1e-5
    assert abs(out[0][2][0] - out[1][2][0]) <= 1e-5 * abs(out[1][2][0])
    assert rel_l2(out[0][2][1], out[1][2][1]) < 1e-4


@pytest.mark.parametrize("variant", ["lie", "nk3_nr3", "phi_store_l2b", "obs_threshold",
                                     "reaction_inv", "sinusoidal"])
def test_gradient_variants_on_own_transforms(variant):
    """J and grad J of the mixed path at 64^3 (the library's own x / y / z transform kernels)
    against the FP64 oracle, over the reference's model and optimiser options: Lie splitting,
    three diffusivity / reaction classes (explicit kappa gradient), stored Phi with the L2b
    regulariser, a thresholded observation operator, reaction inversion, sinusoidal tissue and
    diffusivity."""
    n, nt = 64, 3
    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    d1 = observation(wl, tissue, centers)
    np_ = len(centers)
    o, g = orc(n), gpu(n, MIXED)
    nk = nr = 1
    for ctx in (o, g):
        configure(ctx, wl, tissue, centers)
        ctx.set_obs_filter(np.ones(n ** 3))
        if variant == "lie":
            ctx.set_time(wl.dt, nt, 1)
        elif variant == "nk3_nr3":
            ctx.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=0.2, k_glm_wm=0.1,
                                 r_gm_wm=0.5, r_glm_wm=0.2)
            ctx.set_opt(nk=3, nr=3)
            nk = nr = 3
        elif variant == "phi_store_l2b":
            ctx.set_opt(phi_store=1, regularization_norm=1, beta=0.1)
        elif variant == "obs_threshold":
            ctx.set_obs_threshold(d1, 0.3)
        elif variant == "reaction_inv":
            ctx.set_opt(flag_reaction_inv=1, all_gradients=0)
            ctx.set_c0(o.phi_apply(np.linspace(0.2, 1.0, np_)))
        elif variant == "sinusoidal":
            ctx.set_tissue_sinusoidal()
            ctx.set_diffusivity_sinusoidal(1e-2)
    if nk == 3:
        x = np.concatenate([np.linspace(0.1, 0.9, np_), [wl.kappa, 0.2 * wl.kappa, 0.1 * wl.kappa],
                            [wl.rho, 0.5 * wl.rho, 0.2 * wl.rho]])
    else:
        x = np.concatenate([np.linspace(0.1, 0.9, np_), [wl.kappa, wl.rho]])
    Jo, gro = o.eval_objective_and_gradient(x, d1)
    Jg, grg = g.eval_objective_and_gradient(x, d1)
    assert abs(Jg - Jo) <= 1e-4 * abs(Jo)
    assert rel_l2(grg, gro) < GRAD_TOL


@pytest.mark.parametrize("n", [64, 128, 256])
def test_z_pass_block_order_is_bit_identical(n, monkeypatch):
    """The z pass over its line blocks in descending order (the default) against ascending order
    (GLIA_ZREV=0): every line is transformed on its own, so D apply, state and gradient agree
    bit for bit."""
    nt = 3
    wl, tissue, centers = small_problem(n, nt, n_gauss=8)
    d1 = observation(wl, tissue, centers)
    f = reference_test_field(n) + 0.1 * tissue.wm.reshape(-1)
    x = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    out = []
    for on in ("1", "0"):
        monkeypatch.setenv("GLIA_ZREV", on)
        g = gpu(n, MIXED)
        configure(g, wl, tissue, centers)
        g.set_obs_filter(np.ones(n ** 3))
        c0 = g.phi_apply(np.linspace(0.2, 1.0, len(centers)))
        J, gr = g.eval_objective_and_gradient(x, d1)
        out.append((g.apply_d(f), g.solve_state(c0), J, gr))
        g.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
    assert np.array_equal(out[0][3], out[1][3])
