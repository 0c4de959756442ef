"""The box-local Phi set-up of the CUDA library (k_phi_box, kernels.cuh; set_phi in
engine_impl.cuh) restated in numpy and checked on the CPU against the FP64 oracle's full-grid
construction (Phi::initialize on the grid, the Weierstrass smoother by FFT, Phi::truncate;
src/mat/Phi.cpp:76-144, 238-311): the smoother's periodised Gaussian as three 1-D convolutions
over each function's 5-sigma box widened by Rh = ceil(9.6 s / h) voxels, with the same region
layout, tap order and pass order as the kernel."""
import numpy as np
import pytest

from tests.gpu_common import configure, orc, small_problem


def box_model(n, center, sigma, filt, smoothing_factor=1.0):
    """Returns (lo, values on the box) as k_phi_box computes them (FP64)."""
    h = 2 * np.pi / n
    lo, ext = [], []
    for d in range(3):
        a = (center[d] - 5 * sigma) / h
        b = (center[d] + 5 * sigma) / h
        l, u = int(np.ceil(a - 1e-9)), int(np.floor(b + 1e-9))
        l, u = max(l, 0), min(u, n - 1)
        lo.append(l)
        ext.append(max(0, u - l + 1))
    s = smoothing_factor * 2 * np.pi / n
    Rh = int(np.ceil(9.6 * s / h)) if s > 0 else 0
    assert 2 * Rh + 1 <= n
    if Rh:
        i = np.arange(n)
        w1 = (np.exp((-(i * h) ** 2) / s / s / 2.0)
              + np.exp((-(i * h - 2 * np.pi) ** 2) / s / s / 2.0))
        taps = np.array([w1[d % n] for d in range(-Rh, Rh + 1)]) / w1.sum()
    else:
        taps = np.ones(1)
    # pass 0: f on the widened region, periodic indices, non-periodic distances
    idx = [(np.arange(ext[d] + 2 * Rh) + lo[d] - Rh) % n for d in range(3)]
    X, Y, Z = np.meshgrid(*[ix * h for ix in idx], indexing="ij")
    r = np.sqrt((X - center[0]) ** 2 + (Y - center[1]) ** 2 + (Z - center[2]) ** 2)
    f = np.exp(-(r / (np.sqrt(2.0) * sigma)) ** 2) * filt[np.ix_(*idx)]
    W = 2 * Rh + 1
    # passes 1-3: z, y, x; taps[dd] multiplies the input at local index (box index + dd)
    t1 = sum(taps[dd] * f[:, :, dd:dd + ext[2]] for dd in range(W))
    t2 = sum(taps[dd] * t1[:, dd:dd + ext[1], :] for dd in range(W))
    v = sum(taps[dd] * t2[dd:dd + ext[0], :, :] for dd in range(W))
    bx = [np.arange(lo[d], lo[d] + ext[d]) * h for d in range(3)]
    X, Y, Z = np.meshgrid(*bx, indexing="ij")
    r = np.sqrt((X - center[0]) ** 2 + (Y - center[1]) ** 2 + (Z - center[2]) ** 2)
    return lo, np.where(r / sigma <= 5.0, v, 0.0)


def _compare(o, n, cs, sigma, filt):
    o.set_phi(cs, sigma, 1.0)
    for i, c in enumerate(cs):
        e = np.zeros(len(cs))
        e[i] = 1.0
        full = o.phi_apply(e).reshape(n, n, n)  # phi_i / max(phi_i) (on-the-fly mode)
        lo, v = box_model(n, c, sigma, filt.reshape(n, n, n))
        got = np.zeros((n, n, n))
        got[lo[0]:lo[0] + v.shape[0], lo[1]:lo[1] + v.shape[1], lo[2]:lo[2] + v.shape[2]] = v
        got /= v.max()
        assert np.linalg.norm(got - full) <= 1e-12 * np.linalg.norm(full), i


@pytest.mark.parametrize("n", [32, 64])
def test_box_model_matches_the_oracle_phi(n):
    """The workload's basis: centres on the in-WM lattice of the synthetic brain."""
    wl, tissue, centers = small_problem(n, 2, n_gauss=8)
    o = orc(n)
    configure(o, wl, tissue, centers)
    filt = (((tissue.wm > 0.1) | (tissue.gm > 0.1)) & (tissue.vt < 0.8)).astype(np.float64)
    _compare(o, n, centers, wl.sigma, filt)


def test_box_model_wraps_its_halo_around_the_grid():
    """Uniform tissue (filter 1 everywhere) and centres at the faces and corners of the grid:
    the boxes are clipped, the halos cross the periodic boundary."""
    n = 32
    wl, tissue, centers = small_problem(n, 2, n_gauss=2)
    o = orc(n)
    configure(o, wl, tissue, centers)
    one = np.ones(n ** 3)
    o.set_tissue(one, 0 * one, 0 * one, 0 * one)
    t = 2 * np.pi
    cs = np.array([[0.05, np.pi, t - 0.1], [0.0, 0.0, 0.0], [t - 0.2, t - 0.05, 0.3],
                   [np.pi, 0.1, np.pi]])
    _compare(o, n, cs, wl.sigma, one)


def test_a_basis_function_outside_the_filter_is_negligible():
    """A centre whose whole box lies outside the brain filter: its values on the box are below
    1e-100 of an in-brain function's (the far tails the box-local sum leaves out are of that
    order too), so it adds nothing next to any function centred in the brain; the reference
    would normalise such a near-zero field by its own maximum when it alone is active."""
    n = 32
    wl, tissue, centers = small_problem(n, 2, n_gauss=8)
    filt = (((tissue.wm > 0.1) | (tissue.gm > 0.1)) & (tissue.vt < 0.8)).astype(np.float64)
    _, v = box_model(n, np.array([0.05, np.pi, 2 * np.pi - 0.1]), wl.sigma, filt.reshape(n, n, n))
    _, v_in = box_model(n, centers[0], wl.sigma, filt.reshape(n, n, n))
    assert v.max() < 1e-100 * v_in.max()
