"""Bounded L-BFGS inversion over (p, kappa, rho), the caller of the gradient path.

Restates the reference's optimizer set-up (src/opt/Optimizer.cpp:116-286,
src/opt/TILOptimizer.cpp:245-272, src/opt/TaoInterface.cpp:362-530): TAO BLMVM (bounded
limited-memory variable metric) with 10 correction pairs (lbfgs_vectors_), at most 10 function
evaluations per line search (ls_max_func_evals), stopping when the projected-gradient norm falls
below gttol * ||g_0|| (opttolgrad_ = 1e-3) or below gatol (1e-4), or after newton_maxit (30)
iterations; bounds p >= 0, kappa in [1e-3, 1], rho in [1, 15].

PETSc/TAO (3.7-3.11) is not part of the reference tree; its published algorithms are restated:
- line search (OptimizerSettings::linesearch_, default MT, include/Parameters.h:36): the
  More-Thuente search of MINPACK-2 (dcsrch / dcstep; J. J. More and D. J. Thuente, "Line search
  algorithms with guaranteed sufficient decrease", ACM TOMS 20, 1994) with ftol 1e-4, gtol 0.9,
  xtol 1e-10, minimum step = machine epsilon (ls_minstep_, Optimizer.cpp:153-155), initial step
  1 (:163); on a bounded problem each trial point is projected onto the box and the directional
  derivative is taken along the projected path, g(x_t) . (x_t - x) / t. ARMIJO: projected
  backtracking with sufficient decrease 1e-4 and halving.
- initial inverse Hessian of the two-loop recursion (lbfgs_scale_type_, Optimizer.cpp:180-192 for
  PETSc >= 3.9, default "diagonal"; :225-230 for older PETSc: Broyden scalar scaling with a
  history of 5): "none" (identity), "scalar" (s'y / y'y summed over the last `scale_hist`
  pairs, lbfgs_scale_hist_ = 5), "diagonal" (a diagonal BFGS update of the initial matrix per
  pair, J. C. Gilbert and C. Lemarechal, Math. Programming 45, 1989: with B = D^-1,
  B_i <- B_i + y_i^2 / y's - (B_i s_i)^2 / s'Bs, entries kept positive, started from the scalar
  scaling of the first pair).
The direction is the two-loop product on the gradient, with the variables held at a bound (and
those the step would push out of the box) removed. All vectors are FP64 on the host; each
objective and gradient is one glia_eval_objective[_and_gradient] call.

    python -m glia_gb300.inversion --n 128      # the 128^3 reconstruction, mixed vs FP64
    python -m glia_gb300.inversion --full256 --precisions mixed,fp64,fp64_plain
                                                # the 256^3 one; fp64_plain = the
                                                # reference-structured FP64 engine
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from dataclasses import dataclass, field

import numpy as np

EPS = float(np.finfo(np.float64).eps)


@dataclass
class LbfgsSettings:
    m: int = 10                 # lbfgs_vectors_
    gttol: float = 1e-3         # opttolgrad_: ||g|| < gttol ||g0||
    gatol: float = 1e-4         # gatol_
    maxit: int = 30             # newton_maxit_
    ls_max_funcs: int = 10      # ls_max_func_evals
    line_search: str = "mt"     # linesearch_: "mt" (More-Thuente) or "armijo"
    scale_type: str = "diagonal"  # lbfgs_scale_type_: "none", "scalar", "diagonal"
    scale_hist: int = 5         # lbfgs_scale_hist_
    armijo_c1: float = 1e-4
    shrink: float = 0.5
    mt_ftol: float = 1e-4
    mt_gtol: float = 0.9
    mt_xtol: float = 1e-10
    ls_minstep: float = EPS     # ls_minstep_
    ls_maxstep: float = 1e20


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


# ------------------------------------------------------------------------------------------
# More-Thuente line search (MINPACK-2 dcstep / dcsrch, restated)
# ------------------------------------------------------------------------------------------
def dcstep(stx, fx, dx, sty, fy, dy, stp, fp, dp, brackt, stpmin, stpmax):
    """One safeguarded step of the interval of uncertainty [stx, sty] (cubic / quadratic / secant
    interpolation, four cases). Returns (stx, fx, dx, sty, fy, dy, stp, brackt)."""
    sgnd = dp * np.sign(dx)
    if fp > fx:  # 1: higher value, the minimum is bracketed
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * np.sqrt(max(0.0, (theta / s) ** 2 - (dx / s) * (dp / s)))
        if stp < stx:
            gamma = -gamma
        p = (gamma - dx) + theta
        q = ((gamma - dx) + gamma) + dp
        stpc = stx + (p / q) * (stp - stx)
        stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx)
        stpf = stpc if abs(stpc - stx) < abs(stpq - stx) else stpc + (stpq - stpc) / 2.0
        brackt = True
    elif sgnd < 0.0:  # 2: lower value, derivatives of opposite sign
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * np.sqrt(max(0.0, (theta / s) ** 2 - (dx / s) * (dp / s)))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = ((gamma - dp) + gamma) + dx
        stpc = stp + (p / q) * (stx - stp)
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
        brackt = True
    elif abs(dp) < abs(dx):  # 3: lower value, same sign, derivative decreases in magnitude
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * np.sqrt(max(0.0, (theta / s) ** 2 - (dx / s) * (dp / s)))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = (gamma + (dx - dp)) + gamma
        r = p / q
        if r < 0.0 and gamma != 0.0:
            stpc = stp + r * (stx - stp)
        elif stp > stx:
            stpc = stpmax
        else:
            stpc = stpmin
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        if brackt:
            stpf = stpc if abs(stpc - stp) < abs(stpq - stp) else stpq
            if stp > stx:
                stpf = min(stp + 0.66 * (sty - stp), stpf)
            else:
                stpf = max(stp + 0.66 * (sty - stp), stpf)
        else:
            stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
            stpf = min(stpmax, max(stpmin, stpf))
    else:  # 4: lower value, same sign, derivative does not decrease
        if brackt:
            theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp
            s = max(abs(theta), abs(dy), abs(dp))
            gamma = s * np.sqrt(max(0.0, (theta / s) ** 2 - (dy / s) * (dp / s)))
            if stp > sty:
                gamma = -gamma
            p = (gamma - dp) + theta
            q = ((gamma - dp) + gamma) + dy
            stpf = stp + (p / q) * (sty - stp)
        elif stp > stx:
            stpf = stpmax
        else:
            stpf = stpmin
    if fp > fx:
        sty, fy, dy = stp, fp, dp
    else:
        if sgnd < 0.0:
            sty, fy, dy = stx, fx, dx
        stx, fx, dx = stp, fp, dp
    return stx, fx, dx, sty, fy, dy, stpf, brackt


def more_thuente(phi, f0, g0, stp, s: LbfgsSettings):
    """MINPACK-2 dcsrch: a step satisfying f(t) <= f0 + ftol t g0 and |f'(t)| <= gtol |g0|.
    phi(t) -> (f, f'(t), payload). Returns (t, f, payload, evaluations, converged); payload is
    that of the returned step (None when no evaluation was kept)."""
    xtrapl, xtrapu = 1.1, 4.0
    ftol, gtol, xtol = s.mt_ftol, s.mt_gtol, s.mt_xtol
    stpmin, stpmax = s.ls_minstep, s.ls_maxstep
    if g0 >= 0.0:
        return 0.0, f0, None, 0, False
    brackt, stage = False, 1
    gtest = ftol * g0
    width = stpmax - stpmin
    width1 = 2.0 * width
    stx, fx, gx = 0.0, f0, g0
    sty, fy, gy = 0.0, f0, g0
    stmin, stmax = 0.0, stp + xtrapu * stp
    best = (0.0, f0, None)
    for nfev in range(1, s.ls_max_funcs + 1):
        stp = min(max(stp, stpmin), stpmax)
        f, g, payload = phi(stp)
        ftest = f0 + stp * gtest
        if f <= ftest and f < best[1]:
            best = (stp, f, payload)
        if stage == 1 and f <= ftest and g >= 0.0:
            stage = 2
        if f <= ftest and abs(g) <= gtol * (-g0):
            return stp, f, payload, nfev, True
        if (brackt and (stp <= stmin or stp >= stmax)) or (brackt and stmax - stmin <= xtol * stmax) \
                or (stp == stpmax and f <= ftest and g <= gtest) \
                or (stp == stpmin and (f > ftest or g >= gtest)):
            break  # rounding errors, interval below xtol, or a step bound reached
        if stage == 1 and f <= fx and f > ftest:  # modified function psi(t) = f(t) - f0 - t gtest
            fm, fxm, fym = f - stp * gtest, fx - stx * gtest, fy - sty * gtest
            gm, gxm, gym = g - gtest, gx - gtest, gy - gtest
            stx, fxm, gxm, sty, fym, gym, stp, brackt = dcstep(stx, fxm, gxm, sty, fym, gym, stp,
                                                                fm, gm, brackt, stmin, stmax)
            fx, fy = fxm + stx * gtest, fym + sty * gtest
            gx, gy = gxm + gtest, gym + gtest
        else:
            stx, fx, gx, sty, fy, gy, stp, brackt = dcstep(stx, fx, gx, sty, fy, gy, stp, f, g,
                                                            brackt, stmin, stmax)
        if brackt:
            if abs(sty - stx) >= 0.66 * width1:
                stp = stx + 0.5 * (sty - stx)
            width1 = width
            width = abs(sty - stx)
            stmin, stmax = min(stx, sty), max(stx, sty)
        else:
            stmin = stp + xtrapl * (stp - stx)
            stmax = stp + xtrapu * (stp - stx)
        stp = min(max(stp, stpmin), stpmax)
        if (brackt and (stp <= stmin or stp >= stmax)) or (brackt and stmax - stmin <= xtol * stmax):
            stp = stx
    # no step met both conditions: keep the best sufficient-decrease step, if any
    t, f, payload = best
    return t, f, payload, nfev, False


# ------------------------------------------------------------------------------------------
# L-BFGS initial inverse Hessian
# ------------------------------------------------------------------------------------------
class InitialScaling:
    """H0 of the two-loop recursion: identity, scalar (s'y / y'y over the last `hist` pairs) or
    diagonal (Gilbert-Lemarechal diagonal BFGS update of B0 = H0^-1, per accepted pair)."""

    def __init__(self, kind: str, n: int, hist: int):
        if kind not in ("none", "scalar", "diagonal"):
            raise ValueError(f"unknown scale type {kind}")
        self.kind, self.hist = kind, max(1, hist)
        self.pairs = []
        self.B = None  # diagonal of the initial Hessian (diagonal kind)
        self.n = n

    def update(self, sv, yv):
        self.pairs.append((float(sv @ yv), float(yv @ yv)))
        self.pairs = self.pairs[-self.hist:]
        if self.kind != "diagonal":
            return
        sy = float(sv @ yv)
        if self.B is None:
            self.B = np.full(self.n, float(yv @ yv) / sy)  # start at the scalar scaling
        sBs = float(sv @ (self.B * sv))
        newB = self.B + yv * yv / sy - (self.B * sv) ** 2 / sBs
        ok = np.isfinite(newB) & (newB > 1e-12 * np.max(self.B))
        self.B = np.where(ok, newB, self.B)

    def reset(self):
        self.pairs.clear()
        self.B = None

    def apply(self, q, gnorm):
        if not self.pairs:  # no curvature yet: a step of unit length along the gradient
            return q / max(gnorm, 1e-300)
        if self.kind == "none":
            return q.copy()
        if self.kind == "scalar":
            return q * (sum(p[0] for p in self.pairs) / sum(p[1] for p in self.pairs))
        return q / self.B


def bounded_lbfgs(fun_grad, fun, x0, lb, ub, s: LbfgsSettings = LbfgsSettings()) -> LbfgsResult:
    """Minimise fun over lb <= x <= ub. fun_grad(x) -> (J, g); fun(x) -> J."""
    x = np.clip(np.asarray(x0, dtype=np.float64), lb, ub)
    J, g = fun_grad(x)
    fevals = gevals = 1
    pg = projected_gradient(x, g, lb, ub)
    g0 = float(np.linalg.norm(pg)) or 1.0
    S, Y = [], []
    H0 = InitialScaling(s.scale_type, x.size, s.scale_hist)
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
        r = H0.apply(q, gn)
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
            H0.reset()
            d = -pg / max(gn, 1e-300)
        if s.line_search == "mt":
            def phi(t):
                xt = np.clip(x + t * d, lb, ub)
                Jt, gt = fun_grad(xt)
                return Jt, float(gt @ (xt - x)) / t, (xt, Jt, gt)

            step, Jn, payload, nfev, ok = more_thuente(phi, J, float(g @ d), 1.0, s)
            fevals += nfev
            gevals += nfev
            accepted = payload is not None and Jn < J
            if accepted:
                xn, Jn, gnew = payload
        else:
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
            if accepted and gnew is None:
                Jn, gnew = fun_grad(xn)
                fevals += 1
                gevals += 1
        if not accepted:
            reason = "linesearch"
            break
        sv, yv = xn - x, gnew - g
        if sv @ yv > 1e-12 * np.linalg.norm(sv) * np.linalg.norm(yv):
            S.append(sv)
            Y.append(yv)
            H0.update(sv, yv)
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
                       problem=None, gatol=0.0, progress=False):
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
        if name not in ("mixed", "fp64", "fp64_plain"):
            raise ValueError(f"unknown arm {name} (mixed, fp64, fp64_plain)")
        prec = _abi.GLIA_MIXED if name == "mixed" else _abi.GLIA_FP64
        # fp64_plain: the reference-structured FP64 engine with the full time history (the plain
        # FP64 GPU path); the other arms are the fused engine with checkpoints
        plain = name == "fp64_plain"
        ctx = Context(api, wl.n, prec, _abi.GLIA_ENGINE_REFERENCE if plain else
                      _abi.GLIA_ENGINE_FUSED)
        syn.setup_context(ctx, wl, tissue, centers,
                          _abi.GLIA_HISTORY_FULL if plain else _abi.GLIA_HISTORY_CHECKPOINT,
                          0 if plain else every)
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
        if progress:  # each arm as soon as it ends (a long run cut short keeps the arms done)
            print(json.dumps({name: out[name]}), file=sys.stderr, flush=True)
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
                                        maxit=a.maxit, problem=prob, gatol=a.gatol,
                                        progress=True)))
