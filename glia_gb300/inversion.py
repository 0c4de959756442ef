"""Bounded L-BFGS inversion over (p, kappa, rho), the caller of the gradient path.

Restates the reference's optimizer set-up (src/opt/Optimizer.cpp:116-286,
src/opt/TILOptimizer.cpp:245-272, src/opt/TaoInterface.cpp:362-530): TAO BLMVM (bounded
limited-memory variable metric) with 10 correction pairs, at most 10 function evaluations per line
search, stopping when the projected-gradient norm falls below gttol * ||g_0|| (gttol = 1e-3) or
below gatol (1e-4), or after newton_maxit (30) iterations; bounds p >= 0, kappa in [1e-3, 1],
rho in [1, 15]. The search direction is the two-loop L-BFGS product with the scalar initial
scaling s'y / y'y, projected onto the free variables; the step is a projected backtracking
(Armijo) line search along P(x + a d). All vectors are FP64 on the host; each objective and
gradient is one glia_eval_objective[_and_gradient] call.

    python -m glia_gb300.inversion --n 128      # the 128^3 reconstruction, mixed vs FP64
"""
from __future__ import annotations

import argparse
import json
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class LbfgsSettings:
    m: int = 10                 # lbfgs_vectors_
    gttol: float = 1e-3         # opttolgrad_: ||g|| < gttol ||g0||
    gatol: float = 1e-4         # gatol_
    maxit: int = 30             # newton_maxit_
    ls_max_funcs: int = 10      # ls_max_func_evals
    armijo_c1: float = 1e-4
    shrink: float = 0.5


@dataclass
class LbfgsResult:
    x: np.ndarray
    J: float
    gnorm: float
    gnorm0: float
    iterations: int
    fevals: int
    gevals: int
    reason: str
    history: list = field(default_factory=list)


def projected_gradient(x, g, lb, ub):
    pg = g.copy()
    pg[(x <= lb) & (g > 0)] = 0.0
    pg[(x >= ub) & (g < 0)] = 0.0
    return pg


def bounded_lbfgs(fun_grad, fun, x0, lb, ub, s: LbfgsSettings = LbfgsSettings()) -> LbfgsResult:
    """Minimise fun over lb <= x <= ub. fun_grad(x) -> (J, g); fun(x) -> J."""
    x = np.clip(np.asarray(x0, dtype=np.float64), lb, ub)
    J, g = fun_grad(x)
    fevals = gevals = 1
    pg = projected_gradient(x, g, lb, ub)
    g0 = float(np.linalg.norm(pg)) or 1.0
    S, Y = [], []
    hist = [{"it": 0, "J": J, "gnorm": g0}]
    reason = "maxit"
    it = 0
    for it in range(1, s.maxit + 1):
        gn = float(np.linalg.norm(pg))
        if gn < s.gttol * g0:
            reason = "gttol"
            it -= 1
            break
        if gn < s.gatol:
            reason = "gatol"
            it -= 1
            break
        # two-loop recursion on the projected gradient
        q = pg.copy()
        alphas = []
        for sv, yv in reversed(list(zip(S, Y))):
            rho = 1.0 / (yv @ sv)
            a = rho * (sv @ q)
            q -= a * yv
            alphas.append((rho, a))
        gamma = (S[-1] @ Y[-1]) / (Y[-1] @ Y[-1]) if S else 1.0 / max(gn, 1e-300)
        r = gamma * q
        for (sv, yv), (rho, a) in zip(zip(S, Y), reversed(alphas)):
            b = rho * (yv @ r)
            r += (a - b) * sv
        d = -r
        # variables held at a bound by the gradient, or that the step would push out of the box
        binding = ((x <= lb) & (g > 0)) | ((x >= ub) & (g < 0))
        active = binding | ((x <= lb) & (d < 0)) | ((x >= ub) & (d > 0))
        d[active] = 0.0
        if not d @ pg < 0:  # not a descent direction: restart from the projected gradient
            S.clear()
            Y.clear()
            d = -pg / max(gn, 1e-300)
        # projected backtracking line search; the first trial also takes the gradient (it is
        # accepted in most iterations), later trials take the objective only
        step, accepted, gnew = 1.0, False, None
        for trial in range(s.ls_max_funcs):
            xn = np.clip(x + step * d, lb, ub)
            if trial == 0:
                Jn, gnew = fun_grad(xn)
                gevals += 1
            else:
                Jn, gnew = fun(xn), None
            fevals += 1
            if Jn <= J + s.armijo_c1 * (g @ (xn - x)):
                accepted = True
                break
            step *= s.shrink
        if not accepted:
            reason = "linesearch"
            break
        if gnew is None:
            Jn, gnew = fun_grad(xn)
            fevals += 1
            gevals += 1
        sv, yv = xn - x, gnew - g
        if sv @ yv > 1e-12 * np.linalg.norm(sv) * np.linalg.norm(yv):
            S.append(sv)
            Y.append(yv)
            if len(S) > s.m:
                S.pop(0)
                Y.pop(0)
        x, J, g = xn, Jn, gnew
        pg = projected_gradient(x, g, lb, ub)
        hist.append({"it": it, "J": J, "gnorm": float(np.linalg.norm(pg)), "step": step})
    return LbfgsResult(x=x, J=J, gnorm=float(np.linalg.norm(pg)), gnorm0=g0, iterations=it,
                       fevals=fevals, gevals=gevals, reason=reason, history=hist)


def reference_bounds(np_: int, k_lb=1e-3, k_ub=1.0, rho_lb=1.0, rho_ub=15.0):
    """TILOptimizer::setVariableBounds / RDOptimizer bounds for x = [p, kappa, rho]."""
    lb = np.concatenate([np.zeros(np_), [k_lb, rho_lb]])
    ub = np.concatenate([np.full(np_, np.inf), [k_ub, rho_ub]])
    return lb, ub


def invert(ctx, d1, x0, lb, ub, settings: LbfgsSettings = LbfgsSettings(),
           grad_scale=None) -> LbfgsResult:
    """L-BFGS on a configured context (objective = DerivativeOperatorsRD with all_gradients).
    grad_scale: the k_scale / rho_scale factors of x. The reference's adjoint gradient is taken
    with respect to kappa and rho themselves, so the gradient with respect to the scaled unknowns
    is that gradient times the scale (chain rule)."""
    gs = 1.0 if grad_scale is None else np.asarray(grad_scale, dtype=np.float64)

    def fg(x):
        J, g = ctx.eval_objective_and_gradient(x, d1)
        return J, g * gs

    return bounded_lbfgs(fg, lambda x: ctx.eval_objective(x, d1), x0, lb, ub, settings)


# ------------------------------------------------------------------------------------------
def reconstruction_problem(n=128, nt=40, seed_truth=4, seed_noise=5):
    """The 128^3 reconstruction: 216 Gaussians on the reference's even 6x6x6 lattice (spacing
    1.5 sigma around (pi, pi, pi)), truth with 3 active Gaussians (U[0.5, 1]), rho = 12,
    kappa = 0.03, dt = 0.01, data = forward + N(0, 0.01^2)."""
    from . import synthetic as syn
    from .context import phi_mesh
    from .native import load

    tissue = syn.make_tissue(n, 0)
    sigma = 2 * np.pi / 64
    centers = phi_mesh(load(), 216, [np.pi, np.pi, np.pi], sigma, 1.5)
    rng = np.random.default_rng(seed_truth)
    p = np.zeros(216)
    act = rng.choice(216, size=3, replace=False)
    p[act] = rng.uniform(0.5, 1.0, size=3)
    wl = syn.GradientWorkload(n=n, nt=nt, n_gauss=216, rho=12.0, kappa=0.03)
    return wl, tissue, centers, np.concatenate([p, [wl.kappa, wl.rho]]), seed_noise


def reconstruction_256(n=256, nt=100, n_gauss=1000, seed_truth=6):
    """The 256^3 reconstruction: 1000 Gaussians (sigma = 2pi/64) at the first in-brain lattice
    points, truth with 5 active, rho = 10, kappa = 0.05, dt = 0.01, nt = 100."""
    from . import synthetic as syn

    tissue = syn.make_tissue(n, 0)
    centers = syn.lattice_centers_in_mask(tissue.mask, n_gauss)
    rng = np.random.default_rng(seed_truth)
    p = np.zeros(n_gauss)
    act = rng.choice(n_gauss, size=5, replace=False)
    p[act] = rng.uniform(0.5, 1.0, size=5)
    wl = syn.GradientWorkload(n=n, nt=nt, n_gauss=n_gauss, rho=10.0, kappa=0.05)
    return wl, tissue, centers, np.concatenate([p, [wl.kappa, wl.rho]]), 7


def run_reconstruction(n=128, nt=40, precisions=("mixed", "fp64"), every=10, maxit=100,
                       problem=None, gatol=0.0):
    """L-BFGS from p = 0, kappa and rho at half their true values, to a 1e-3 relative reduction
    of the projected gradient (gatol = 0: the relative test alone, as the workload states; the
    reference's default adds gatol = 1e-4). kappa and rho enter x through the reference's
    k_scale_ / rho_scale_ (x_kappa = kappa / 0.01, x_rho = rho / 10) so that all unknowns are
    O(1). Each arm also reports the relative L2 error of its final state c(1) against an FP64
    forward at the arm's own final parameters."""
    from . import _abi
    from . import synthetic as syn
    from .context import Context
    from .native import load

    wl, tissue, centers, x_true, seed_noise = problem or reconstruction_problem(n, nt)
    npp = len(centers)
    k_scale, rho_scale = 1e-2, 10.0
    scale = np.concatenate([np.ones(npp), [k_scale, rho_scale]])
    api = load()
    out = {"n": wl.n, "nt": wl.nt, "np": npp, "x_true_active": int(np.count_nonzero(x_true[:npp])),
           "k_scale": k_scale, "rho_scale": rho_scale}
    data = None
    for name in precisions:
        prec = _abi.GLIA_MIXED if name == "mixed" else _abi.GLIA_FP64
        ctx = Context(api, wl.n, prec)
        syn.setup_context(ctx, wl, tissue, centers, _abi.GLIA_HISTORY_CHECKPOINT, every)
        ctx.set_opt(k_scale=k_scale, rho_scale=rho_scale)
        ctx.set_obs_filter(np.ones(wl.n ** 3))
        if data is None:  # data from the FP64 forward at the true parameters
            gen = Context(api, wl.n, _abi.GLIA_FP64)
            syn.setup_context(gen, wl, tissue, centers, _abi.GLIA_HISTORY_FULL, 0)
            gen.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
            c1 = gen.solve_state(gen.phi_apply(x_true[:npp]))
            data = c1 + np.random.default_rng(seed_noise).normal(0.0, 0.01, c1.size)
            gen.close()
        lb, ub = reference_bounds(npp)
        lb, ub = lb / scale, ub / scale
        x0 = np.concatenate([np.zeros(npp), [0.5 * wl.kappa, 0.5 * wl.rho]]) / scale
        t0 = time.perf_counter()
        res = invert(ctx, data, x0, lb, ub, LbfgsSettings(maxit=maxit, gatol=gatol),
                     grad_scale=scale)
        wall = time.perf_counter() - t0
        x = res.x * scale
        # final state of this arm vs an FP64 forward at the same parameters
        ctx.set_coefficients(k=float(x[npp]), rho=float(x[npp + 1]), k_gm_wm=wl.k_gm_wm)
        c_arm = ctx.solve_state(ctx.phi_apply(x[:npp]))
        chk = Context(api, wl.n, _abi.GLIA_FP64)
        syn.setup_context(chk, wl, tissue, centers, _abi.GLIA_HISTORY_CHECKPOINT, every)
        chk.set_coefficients(k=float(x[npp]), rho=float(x[npp + 1]), k_gm_wm=wl.k_gm_wm)
        c_ref = chk.solve_state(chk.phi_apply(x[:npp]))
        chk.close()
        state_err = float(np.linalg.norm(c_arm - c_ref) / np.linalg.norm(c_ref))
        err_p = float(np.linalg.norm(x[:npp] - x_true[:npp]) / np.linalg.norm(x_true[:npp]))
        out[name] = {"wall_s": wall, "s_per_eval": wall / max(1, res.gevals),
                     "final_state_rel_err_vs_fp64": state_err,
                     "iterations": res.iterations, "fevals": res.fevals,
                     "gevals": res.gevals, "reason": res.reason, "J": res.J,
                     "gnorm_rel": res.gnorm / res.gnorm0, "p_rel_err": err_p,
                     "kappa": float(x[npp]), "kappa_rel_err": abs(x[npp] / x_true[npp] - 1),
                     "rho": float(x[npp + 1]), "rho_rel_err": abs(x[npp + 1] / x_true[npp + 1] - 1)}
        ctx.close()
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--nt", type=int, default=40)
    ap.add_argument("--precisions", default="mixed,fp64")
    ap.add_argument("--maxit", type=int, default=100)
    ap.add_argument("--gatol", type=float, default=0.0)
    ap.add_argument("--full256", action="store_true",
                    help="the 256^3 reconstruction with 1000 Gaussians (nt = 100)")
    a = ap.parse_args()
    prob = reconstruction_256() if a.full256 else None
    print(json.dumps(run_reconstruction(a.n, a.nt, tuple(a.precisions.split(",")),
                                        maxit=a.maxit, problem=prob, gatol=a.gatol)))
