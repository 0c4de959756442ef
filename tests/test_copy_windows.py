"""The bulk-copy windows of the y-inverse pass (k_yinv_bulk, ownfft.cuh) on the CPU: for every
tile and row at n = 64, 128, 256, the copied window of T + 2 complex starting one complex early on
odd rows (rows are n/2 + 1 complex long, 8-byte aligned only) must start 16-byte aligned in
global and shared memory, be a multiple of 16 bytes long, and stay inside the 3-field buffer the
G arrays live in. The formulas restate the kernel's address arithmetic; the tile widths T are
YDecomp's."""
import numpy as np
import pytest

TILE = {64: 32, 128: 32, 256: 16}  # YDecomp<n>::T


@pytest.mark.parametrize("n", [64, 128, 256])
def test_row_windows_are_aligned_and_in_bounds(n):
    T = TILE[n]
    nq, nh = n // 2, n // 2 + 1
    cb_count = nq // T
    ps = n * nh                      # complex per x plane
    ns = n * ps                      # complex per half spectrum (G_x; G_0 follows it)
    ts = T + 2                       # window length (complex)
    buffer_bytes = 3 * n ** 3 * 4    # g3r_: three FP32 fields
    x = np.arange(n)[:, None, None]
    cb = np.arange(cb_count)[None, :, None]
    r = np.arange(n)[None, None, :]
    for g in (0, 1):                 # G_x, then G_0 = G_x + ns
        start = (g * ns + x * ps + r * nh + cb * T - (r & 1)) * 8
        assert np.all(start % 16 == 0)
        assert np.all(start >= 0)
        assert np.all(start + ts * 8 <= buffer_bytes)
    assert (ts * 8) % 16 == 0
    dst = np.arange(n) * ts * 8      # slot + r * TS (complex) in shared memory
    assert np.all(dst % 16 == 0)
    # the window holds columns kz0 - (r & 1) ... kz0 + T: the tile's T columns are inside it
    assert np.all((r & 1) + T <= ts)


@pytest.mark.parametrize("n", [64, 128, 256])
def test_windows_cover_each_tile_exactly_once(n):
    """Every (x, ky, kz < n/2) element of a G array is read by exactly one tile (as one of the
    window's T columns at offset (r & 1))."""
    T = TILE[n]
    nq, nh = n // 2, n // 2 + 1
    seen = np.zeros((n, nh), dtype=np.int64)   # one x plane suffices: tiles repeat per plane
    for cb in range(nq // T):
        for r in range(n):
            cols = cb * T + np.arange(T)
            seen[r, cols] += 1
    assert np.all(seen[:, :nq] == 1) and np.all(seen[:, nq] == 0)  # kz = n/2 comes via cp.async
