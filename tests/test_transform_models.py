"""numpy models of the own-transform D apply (CPU): the algebra the FP32 kernels follow, checked
against numpy's FFT.

- The pipeline: x inverse into two arrays (G_x, G_0), y inverse with the kz = 0 / n/2 columns
  packed into one complex column, the z pass on two real lines per complex transform (H_x with
  H_y of a line, H_0 of two neighbouring lines), y forward with unpacking, x forward with the
  divergence — against the direct spectral D u = div(k grad u) with Nyquist wave numbers zeroed
  (k_xinv, k_yinv_bulk, k_zpass2, k_yfwd, k_xfwd_own).
- The z pair transform at the thread level of k_zpass2 (n = R1 x R2 with R2 threads per line,
  R1-point DFTs over a at index R2 a + t, twiddles w^(t k1), R2-point DFTs over the thread's rows
  t + R2 ii, the inverse's output order used as the forward's input order, the split by Hermitian
  symmetry) for the three decompositions the kernel instantiates.
"""
import numpy as np
import pytest


def _wn(k, n):
    k = np.asarray(k)
    return np.where(k < n // 2, k, np.where(k == n // 2, 0, k - n))


def _finv(a, ax):  # unnormalised inverse DFT along ax
    return np.fft.ifft(a, axis=ax) * a.shape[ax]


def _pair_line(A, B, ka, kb, n):
    """Two real lines from packed half spectra A, B (slot 0 = (X[0], X[n/2]) as re / im):
    z = a + i b through one inverse transform, times (ka, kb), forward, split. Returns the packed
    half spectra of ka a and kb b."""
    nq = n // 2

    def full(S):
        X = np.zeros(n, complex)
        X[0], X[nq] = S[0].real, S[0].imag
        X[1:nq] = S[1:]
        X[nq + 1:] = np.conj(S[1:][::-1])
        return X

    z = _finv(full(A) + 1j * full(B), 0)
    zp = ka * z.real + 1j * kb * z.imag
    Z = np.fft.fft(zp)
    Zm = np.conj(Z[(-np.arange(n)) % n])
    Ap, Bp = (Z + Zm) / 2, (Z - Zm) / 2j
    out = []
    for Y in (Ap, Bp):
        S = Y[:nq].copy()
        S[0] = Y[0].real + 1j * Y[nq].real
        out.append(S)
    return out


def test_pipeline_model_matches_the_direct_spectral_d_apply():
    n = 16
    nh, nq, N = n // 2 + 1, n // 2, n ** 3
    rng = np.random.default_rng(0)
    kf = rng.random((n, n, n)) + 0.5
    u = rng.standard_normal((n, n, n))
    uh = np.fft.rfftn(u)
    wx = _wn(np.arange(n), n)[:, None, None]
    wy = _wn(np.arange(n), n)[None, :, None]
    wz = _wn(np.arange(nh), n)[None, None, :]
    grads = [np.fft.irfftn(1j * w * uh, s=(n, n, n), axes=(0, 1, 2)) for w in (wx, wy, wz)]
    ref = sum(1j * w * np.fft.rfftn(kf * g) for w, g in zip((wx, wy, wz), grads))
    # x inverse: two arrays (the y and z multipliers are constant along x)
    G0 = _finv(uh, 0) / N
    Gx = _finv(1j * wx * uh, 0) / N

    def pack(G):  # kz = 0 and kz = n/2 as one column A + iB
        P = G[:, :, :nq].copy()
        P[:, :, 0] = G[:, :, 0] + 1j * G[:, :, nq]
        return P

    Hx, H0 = _finv(pack(Gx), 1), _finv(pack(G0), 1)
    Hy = _finv(1j * wy * pack(G0), 1)
    # z pass: (H_x, H_y) of a line as one pair; H_0 with i w_z on both sides, lines in pairs
    wq = _wn(np.arange(nq), n)
    Kx, Ky, Lz = (np.zeros_like(Hx) for _ in range(3))
    for x in range(n):
        for y in range(n):
            Kx[x, y], Ky[x, y] = _pair_line(Hx[x, y], Hy[x, y], kf[x, y], kf[x, y], n)
        for y in range(0, n, 2):
            D0, D1 = 1j * wq * H0[x, y], 1j * wq * H0[x, y + 1]
            A, B = _pair_line(D0, D1, kf[x, y], kf[x, y + 1], n)
            Lz[x, y], Lz[x, y + 1] = 1j * wq * A, 1j * wq * B
    # y forward and unpacking of the kz = 0 / n/2 column
    Mx = np.fft.fft(Kx, axis=1)
    Mr = 1j * wy * np.fft.fft(Ky, axis=1) + np.fft.fft(Lz, axis=1)

    def unpack(M):
        U = np.zeros((n, n, nh), complex)
        U[:, :, 1:nq] = M[:, :, 1:]
        Z = M[:, :, 0]
        Zm = np.conj(Z[:, (-np.arange(n)) % n])
        U[:, :, 0], U[:, :, nq] = (Z + Zm) / 2, (Z - Zm) / 2j
        return U

    out = 1j * wx * np.fft.fft(unpack(Mx), axis=0) + np.fft.fft(unpack(Mr), axis=0)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def _dft(v, sign):
    j = np.arange(len(v))
    return np.exp(sign * 2j * np.pi * np.outer(j, j) / len(v)) @ v


@pytest.mark.parametrize("n,R1,R2", [(64, 8, 8), (128, 16, 8), (256, 16, 16)])
def test_zpass2_thread_decomposition(n, R1, R2):
    nq, KPT = n // 2, R1 // R2
    rng = np.random.default_rng(n)
    A = rng.standard_normal(nq) + 1j * rng.standard_normal(nq)
    B = rng.standard_normal(nq) + 1j * rng.standard_normal(nq)
    ka, kb = rng.uniform(0.1, 1.0, n), rng.uniform(0.1, 1.0, n)
    want = _pair_line(A, B, ka, kb, n)

    def Zin(k):  # the kernel's pre-processing of a packed pair
        if k == 0:
            return A[0].real + 1j * B[0].real
        if k == nq:
            return A[0].imag + 1j * B[0].imag
        if k < nq:
            return A[k] + 1j * B[k]
        return np.conj(A[n - k]) + 1j * np.conj(B[n - k])

    W = lambda e, s: np.exp(s * 2j * np.pi * e / n)
    E = np.zeros((R1, R2), complex)
    for t in range(R2):  # stage 1 of the inverse, twiddles, exchange
        u = _dft(np.array([Zin(R2 * a + t) for a in range(R1)]), +1)
        E[:, t] = u * W(t * np.arange(R1), +1)
    v = {}
    for t in range(R2):  # stage 2 on the thread's rows, times k
        for ii in range(KPT):
            col = _dft(E[t + R2 * ii, :], +1)
            for k2 in range(R2):
                p = t + R2 * ii + R1 * k2
                v[t, ii, k2] = ka[p] * col[k2].real + 1j * kb[p] * col[k2].imag
    E = np.zeros((R1, R2), complex)
    for t in range(R2):  # forward: the thread holds z'[R2 a + t] at a = ii + KPT k2
        u = np.zeros(R1, complex)
        for ii in range(KPT):
            for k2 in range(R2):
                assert t + R2 * ii + R1 * k2 == R2 * (ii + KPT * k2) + t
                u[ii + KPT * k2] = v[t, ii, k2]
        E[:, t] = _dft(u, -1) * W(t * np.arange(R1), -1)
    Z = np.zeros(n, complex)
    for t in range(R2):
        for ii in range(KPT):
            Z[t + R2 * ii + R1 * np.arange(R2)] = _dft(E[t + R2 * ii, :], -1)
    Zm = np.conj(Z[(-np.arange(n)) % n])
    Ap, Bp = (Z + Zm) / 2, (Z - Zm) / 2j
    for Y, S in zip((Ap, Bp), want):
        got = Y[:nq].copy()
        got[0] = Y[0].real + 1j * Y[nq].real
        assert np.abs(got - S).max() <= 1e-12 * np.abs(S).max()
