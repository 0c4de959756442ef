"""Data preprocessing in front of the inversion: data-driven Gaussian centres and the
edema-based observation mask.

`data_driven_centers` is Phi::setGaussians(Vec data) (src/mat/Phi.cpp:615-1004) for one process
(the whole grid local, no neighbour exchange): on the lattice of points X with
fmod(X, space) == 0, space = spacing_factor * sigma / h voxels, a centre is kept when more than
gaussian_vol_frac * (lattice points of the ball) voxels of the ball of radius sigma / h around it
hold data above data_threshold (checkTumorExistence / ...OutOfProc, :457-520; the ball is clipped
to the domain, not wrapped). The reference's loop arithmetic is kept: lattice coordinates advance
by `x += space` on an integer (so a fractional spacing advances by its truncation after the first
point) and the ball's index range is [x - r, x + r] truncated toward zero.
"""
from __future__ import annotations

import math

import numpy as np


def _trunc(v: float) -> int:
    return int(v)  # C conversion of a float to int: toward zero


def ball_offsets(radius: float):
    """Integer offsets (i, j, k), |(i, j, k)| <= radius, over the reference's loop range."""
    lo, hi = _trunc(-radius), _trunc(radius)
    out = []
    for i in range(lo, hi + 1):
        for j in range(lo, hi + 1):
            for k in range(lo, hi + 1):
                if math.sqrt(i * i + j * j + k * k) <= radius:
                    out.append((i, j, k))
    return out


def lattice_axis(n: int, space: float):
    """Lattice coordinates along one axis: from the first to the last index with
    fmod(index, space) == 0, advancing by `x += space` on an integer."""
    if space < 1.0:
        raise ValueError("centre spacing below one voxel (the reference's lattice loop would not "
                         "advance)")
    hits = [x for x in range(n) if math.fmod(x, space) == 0.0]
    if not hits:
        return []
    start, end = hits[0], hits[-1]
    xs, x = [], start
    while x <= end:
        xs.append(x)
        x = _trunc(x + space)
    return xs


def data_driven_centers(data: np.ndarray, sigma: float = 2 * np.pi / 256,
                        data_threshold: float = 0.05, gaussian_vol_frac: float = 0.0,
                        spacing_factor: float = 2.0, labels: np.ndarray | None = None):
    """(centres (np, 3) in [0, 2pi), component label per centre, tumour fraction field).

    data: (n, n, n) field (e.g. the observed tumour concentration); labels: optional (n, n, n)
    component labels (Phi::labels_), 1 for every centre when absent."""
    data = np.asarray(data, dtype=np.float64)
    n = data.shape[0]
    if data.shape != (n, n, n):
        raise ValueError("data must be an n^3 field")
    h = 2 * np.pi / n
    radius = sigma / h
    space = spacing_factor * sigma / h
    offs = ball_offsets(radius)
    interior = len(offs)
    axis = lattice_axis(n, space)
    tumor = data > data_threshold
    # count of tumour voxels in the clipped ball around every lattice point
    pts = np.array([(x, y, z) for x in axis for y in axis for z in axis], dtype=np.int64)
    counts = np.zeros(len(pts), dtype=np.int64)
    for (i, j, k) in offs:
        q = pts + np.array([i, j, k])
        ok = np.all((q >= 0) & (q < n), axis=1)
        counts[ok] += tumor[q[ok, 0], q[ok, 1], q[ok, 2]]
    frac = np.zeros((n, n, n))
    frac[pts[:, 0], pts[:, 1], pts[:, 2]] = counts / interior
    keep = counts > gaussian_vol_frac * interior
    sel = pts[keep]
    centers = sel.astype(np.float64) * h
    if labels is not None:
        comp = np.asarray(labels)[sel[:, 0], sel[:, 1], sel[:, 2]].astype(np.int64)
    else:
        comp = np.ones(len(sel), dtype=np.int64)
    return centers, comp, frac


def edema_observation_mask(tc: np.ndarray, ed: np.ndarray, lam: float) -> np.ndarray:
    """createEdemaBasedObservationMask (src/utils/Utils.cpp:567-590): O = 1 on the tumour core
    (tc > 0.99), 0 on edema (ed > 0.99), lam elsewhere; the diagonal of the observation operator
    for glia_set_obs_filter."""
    tc = np.asarray(tc, dtype=np.float64)
    ed = np.asarray(ed, dtype=np.float64)
    return np.where(tc > 0.99, 1.0, np.where(ed > 0.99, 0.0, float(lam)))
