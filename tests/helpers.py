"""Shared inputs for the tests: the reference's own test fields and seeded synthetic inputs."""
from __future__ import annotations

import numpy as np


def grid(n):
    h = 2 * np.pi / n
    X = np.arange(n) * h
    return X[:, None, None], X[None, :, None], X[None, None, :]


def reference_test_field(n):
    """createTestFunction (src/test/helper.cpp:17-45): exp(-(r/R)^2), R = sqrt(2)*2pi/64,
    centred at (pi, pi, pi)."""
    x, y, z = grid(n)
    R = np.sqrt(2.0) * (2 * np.pi) / 64
    r = np.sqrt((x - np.pi) ** 2 + (y - np.pi) ** 2 + (z - np.pi) ** 2)
    return np.exp(-(r / R) ** 2).reshape(-1).copy()


def gaussian_at(n, center, sigma):
    x, y, z = grid(n)
    r2 = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2
    return np.exp(-r2 / (2 * sigma ** 2)).reshape(-1).copy()


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)
