"""Seeded synthetic inputs for the reaction–diffusion workloads (host-side numpy).

Tissue: an ellipsoid brain mask centred at (pi, pi, pi) with semi-axes (0.8pi, 0.7pi, 0.6pi);
an i.i.d. N(0, 1) field (seeded) smoothed by a 2-voxel Gaussian and rescaled to [0, 1] by its
in-mask min/max; WM = [xi > 0.75], GM = [0.45 < xi <= 0.75], CSF = [xi <= 0.45] inside the mask;
each class then smoothed by a 1-voxel Gaussian. The smoother is the reference's Weierstrass
filter (periodised Gaussian with eight images, normalised to unit sum;
src/grad/SpectralOperators.cpp:264-381) evaluated with numpy FFTs. VT = 0.

These stand in for the reference's MRI atlases (the clinical data are not distributed).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * np.pi


def weierstrass_kernel(n: int, sigma: float) -> np.ndarray:
    h = TWO_PI / n
    X = np.arange(n) * h
    Xp = X - TWO_PI

    def g(a):
        return np.exp(-(a * a) / sigma / sigma / 2.0)

    gx = (g(X), g(Xp))
    f = np.zeros((n, n, n))
    for ax in gx:
        for ay in gx:
            for az in gx:
                f += ax[:, None, None] * ay[None, :, None] * az[None, None, :]
    f[np.isnan(f)] = 0.0
    return f / f.sum()


def smooth(field: np.ndarray, sigma: float) -> np.ndarray:
    n = field.shape[0]
    k = weierstrass_kernel(n, sigma)
    return np.fft.irfftn(np.fft.rfftn(k) * np.fft.rfftn(field), s=field.shape, axes=(0, 1, 2))


@dataclass
class Tissue:
    wm: np.ndarray
    gm: np.ndarray
    csf: np.ndarray
    vt: np.ndarray
    mask: np.ndarray

    def flat(self):
        return [a.reshape(-1).astype(np.float64) for a in (self.wm, self.gm, self.csf, self.vt)]


def ellipsoid_mask(n: int) -> np.ndarray:
    h = TWO_PI / n
    X = np.arange(n) * h - np.pi
    a, b, c = 0.8 * np.pi, 0.7 * np.pi, 0.6 * np.pi
    r = (X[:, None, None] / a) ** 2 + (X[None, :, None] / b) ** 2 + (X[None, None, :] / c) ** 2
    return r <= 1.0


def make_tissue(n: int, seed: int = 0) -> Tissue:
    h = TWO_PI / n
    rng = np.random.default_rng(seed)
    mask = ellipsoid_mask(n)
    xi = smooth(rng.standard_normal((n, n, n)), 2.0 * h)
    lo, hi = xi[mask].min(), xi[mask].max()
    xi = (xi - lo) / (hi - lo)
    wm = (mask & (xi > 0.75)).astype(np.float64)
    gm = (mask & (xi > 0.45) & (xi <= 0.75)).astype(np.float64)
    csf = (mask & (xi <= 0.45)).astype(np.float64)
    wm, gm, csf = (smooth(a, 1.0 * h) for a in (wm, gm, csf))
    return Tissue(wm=wm, gm=gm, csf=csf, vt=np.zeros_like(wm), mask=mask)


def lattice_centers_in_mask(region: np.ndarray, count: int) -> np.ndarray:
    """The first `count` points, in x-major order, of the coarsest uniform voxel lattice
    (offset half a spacing) that has at least `count` points inside `region`."""
    n = region.shape[0]
    h = TWO_PI / n
    for s in range(n // 2, 0, -1):
        idx = np.arange(s // 2, n, s)
        pts = [(i, j, k) for i in idx for j in idx for k in idx if region[i, j, k]]
        if len(pts) >= count:
            return np.array(pts[:count], dtype=np.float64) * h
    raise ValueError("region too small for the requested number of centres")


def sparse_coefficients(np_: int, density: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    k = max(1, int(round(density * np_)))
    p = np.zeros(np_)
    act = rng.choice(np_, size=k, replace=False)
    p[act] = rng.uniform(0.0, 1.0, size=k)
    return p


@dataclass
class GradientWorkload:
    """Forward + adjoint gradient evaluation at n^3 (the 256^3, nt = 100 headline case and its
    smaller parity sizes): 512 Gaussians (sigma = 2pi/64) at the first in-WM lattice points,
    p ~ U[0,1] on 5 % of entries, rho = 8, kappa = 0.02 (k = kappa (wm + 0.2 gm), rho(x) = rho wm),
    dt = 0.01, nt = 100; data = the forward result with rho * 1.2, kappa * 0.8 and p re-seeded,
    thresholded at 0.5; O = I, beta = 0."""

    n: int = 256
    nt: int = 100
    dt: float = 0.01
    n_gauss: int = 512
    rho: float = 8.0
    kappa: float = 0.02
    k_gm_wm: float = 0.2
    sigma: float = TWO_PI / 64
    density: float = 0.05
    tissue_seed: int = 0

    def tissue(self) -> Tissue:
        return make_tissue(self.n, self.tissue_seed)

    def centers(self, tissue: Tissue) -> np.ndarray:
        return lattice_centers_in_mask(tissue.wm > 0.5, self.n_gauss)

    def p_true(self) -> np.ndarray:
        return sparse_coefficients(self.n_gauss, self.density, 1)

    def p_obs(self) -> np.ndarray:
        return sparse_coefficients(self.n_gauss, self.density, 2)

    def x_eval(self) -> np.ndarray:
        return np.concatenate([self.p_true(), [self.kappa, self.rho]])

    def x_obs(self) -> np.ndarray:
        return np.concatenate([self.p_obs(), [self.kappa * 0.8, self.rho * 1.2]])


def setup_context(ctx, wl: GradientWorkload, tissue: Tissue, centers: np.ndarray,
                  history_mode: int = 0, every: int = 10):
    """Configures a Context (CUDA library or any library with the same C-ABI) for `wl`."""
    ctx.set_time(wl.dt, wl.nt, 2)
    ctx.set_tissue(*tissue.flat())
    ctx.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    ctx.set_phi(centers, wl.sigma, 1.0)
    ctx.set_opt(np=len(centers), nk=1, nr=1, flag_reaction_inv=0, diffusivity_inversion=1,
                regularization_norm=0, beta=0.0, k_scale=1.0, rho_scale=1.0, phi_store=0,
                all_gradients=1)
    ctx.set_history(history_mode, every, 0)
