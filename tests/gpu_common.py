"""Fixtures shared by the GPU tests: contexts on the CUDA library and on the oracle."""
from __future__ import annotations

import numpy as np

from glia_gb300 import _abi
from glia_gb300.context import Context
from glia_gb300 import native
from oracle import oracle

FP64, MIXED = _abi.GLIA_FP64, _abi.GLIA_MIXED
FUSED, REFERENCE = _abi.GLIA_ENGINE_FUSED, _abi.GLIA_ENGINE_REFERENCE

# tolerances stated by the workload: state rel-L2 <= 1e-5 (FP64) / 1e-4 (mixed), gradient 1e-4
STATE_TOL = {FP64: 1e-5, MIXED: 1e-4}
GRAD_TOL = 1e-4


def gpu(n, precision=FP64, engine=FUSED) -> Context:
    return Context(native.load(), n, precision, engine)


def orc(n) -> Context:
    return oracle.context(n)


def small_problem(n=32, nt=8, n_gauss=8, seed=0):
    from glia_gb300 import synthetic as syn

    wl = syn.GradientWorkload(n=n, nt=nt, n_gauss=n_gauss, tissue_seed=seed)
    tissue = wl.tissue()
    centers = syn.lattice_centers_in_mask(tissue.wm > 0.5, n_gauss)
    return wl, tissue, centers


def configure(ctx, wl, tissue, centers, history=_abi.GLIA_HISTORY_FULL, every=4):
    from glia_gb300 import synthetic as syn

    syn.setup_context(ctx, wl, tissue, centers, history, every)


def observation(wl, tissue, centers):
    """Thresholded forward result with perturbed parameters, computed by the oracle."""
    o = orc(wl.n)
    configure(o, wl, tissue, centers)
    o.set_coefficients(k=wl.kappa * 0.8, rho=wl.rho * 1.2, k_gm_wm=wl.k_gm_wm)
    p = np.zeros(len(centers))
    p[: max(1, len(centers) // 3)] = 0.7
    c0 = o.phi_apply(p)
    c1 = o.solve_state(c0)
    return (c1 > 0.5 * c1.max()).astype(np.float64)
