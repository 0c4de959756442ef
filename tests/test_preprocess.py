"""Data-driven Gaussian centres (glia_gb300/preprocess.py) against a loop-by-loop restatement of
Phi::setGaussians(Vec data) for one process (src/mat/Phi.cpp:615-1004, checkTumorExistence
:457-520) on seeded synthetic tumour data."""
import math

import numpy as np
import pytest

from glia_gb300.preprocess import data_driven_centers, edema_observation_mask, lattice_axis


def _loops(data, sigma, thr, frac, spacing_factor=2.0):
    n = data.shape[0]
    h = 2 * math.pi / n
    r = sigma / h
    space = spacing_factor * sigma / h
    interior = 0
    for i in range(int(-r), int(r) + 1):
        for j in range(int(-r), int(r) + 1):
            for k in range(int(-r), int(r) + 1):
                if math.sqrt(i * i + j * j + k * k) <= r:
                    interior += 1
    idx = [X for X in range(n) if math.fmod(X, space) == 0]
    start, end = idx[0], idx[-1]
    marker = {}
    x = start
    while x <= end:
        y = start
        while y <= end:
            z = start
            while z <= end:
                num = 0
                for i in range(int(x - r), int(x + r) + 1):
                    for j in range(int(y - r), int(y + r) + 1):
                        for k in range(int(z - r), int(z + r) + 1):
                            if not (0 <= i < n and 0 <= j < n and 0 <= k < n):
                                continue
                            d = math.sqrt((i - x) ** 2 + (j - y) ** 2 + (k - z) ** 2)
                            if d <= r and data[i, j, k] > thr:
                                num += 1
                marker[(x, y, z)] = num
                z = int(z + space)
            y = int(y + space)
        x = int(x + space)
    centers = [np.array(p) * h for p in sorted(marker) if marker[p] > frac * interior]
    return np.array(centers).reshape(-1, 3)


def _blobs(n, seed):
    rng = np.random.default_rng(seed)
    g = np.arange(n)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    d = np.zeros((n, n, n))
    for _ in range(3):
        c = rng.uniform(0.2 * n, 0.8 * n, 3)
        d += np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * (0.06 * n) ** 2))
    return d


@pytest.mark.parametrize("r_vox,frac", [(1.0, 0.0), (1.5, 0.2), (2.0, 0.1)])
def test_centres_match_the_loop_restatement(r_vox, frac):
    n = 24
    data = _blobs(n, 3)
    sigma = r_vox * 2 * math.pi / n
    c, comp, field = data_driven_centers(data, sigma, 0.05, frac)
    ref = _loops(data, sigma, 0.05, frac)
    assert len(c) > 0 and c.shape == ref.shape
    assert np.allclose(c, ref, atol=0, rtol=0)
    assert np.all(comp == 1)


def test_component_labels_and_lattice_rules():
    n = 16
    data = _blobs(n, 5)
    lab = np.ones((n, n, n)) * 2
    c, comp, _ = data_driven_centers(data, 2 * math.pi / n, 0.05, 0.0, labels=lab)
    assert np.all(comp == 2)
    # fractional spacing: the first step is the spacing, later ones its truncation
    assert lattice_axis(16, 2.5)[:4] == [0, 2, 4, 6]
    with pytest.raises(ValueError):
        lattice_axis(16, 0.5)


def test_edema_observation_mask():
    tc = np.array([1.0, 0.0, 0.0, 1.0, 0.5])
    ed = np.array([0.0, 1.0, 0.0, 1.0, 0.0])
    assert np.array_equal(edema_observation_mask(tc, ed, 0.3), [1.0, 0.0, 0.3, 1.0, 0.3])


@pytest.mark.parametrize("n,r_vox,frac,sf", [(32, 1.0, 0.0, 2.0), (32, 1.5, 0.2, 2.0),
                                             (64, 2.0, 0.1, 2.0), (32, 2.0, 0.0, 1.5)])
def test_oracle_restatement_matches_numpy(n, r_vox, frac, sf):
    """The FP64 oracle's C++ restatement of the reference's loops (oracle_glia_phi_data_centers)
    and the numpy version give the same centres and the same tumour-fraction field."""
    from oracle import oracle

    data = _blobs(n, 7)
    sigma = r_vox * 2 * math.pi / n
    o = oracle.context(n)
    c_o, f_o = o.phi_data_centers(data.reshape(-1), sigma, 0.05, frac, sf, with_frac=True)
    c_n, _, f_n = data_driven_centers(data, sigma, 0.05, frac, spacing_factor=sf)
    assert len(c_n) > 0
    assert np.array_equal(c_o, c_n)
    assert np.array_equal(f_o.reshape(n, n, n), f_n)


def test_oracle_refuses_bad_centre_settings():
    from glia_gb300.context import GliaError
    from oracle import oracle

    o = oracle.context(16)
    data = np.zeros(16 ** 3)
    with pytest.raises(GliaError):
        o.phi_data_centers(data, 2 * math.pi / 16, 0.05, -0.1)      # negative volume fraction
    with pytest.raises(GliaError):
        o.phi_data_centers(data, 0.1 * 2 * math.pi / 16, 0.05, 0.0)  # spacing below one voxel
