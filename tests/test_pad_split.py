"""Index arithmetic of the register-resident 3/2 padding and truncation y
passes (k_colsr_pad in les_gb300/csrc/fft_kernels.cuh), restated in numpy
and checked against numpy's FFT with the padd / unpadd row maps
(padd.f90:123-133, unpadd.f90:143-155).  No GPU: this pins the algorithm the
kernel implements (the split of both lengths as 16 L, the thread layouts,
the twiddles and the in-register padding map); the GPU tests check the
kernel itself against the FP64 step.
"""
import numpy as np
import pytest


def fwd_16l(V, L):
    """Thread r < L holds x[r + L n2] (n2 < 16) -> thread r < 16 holds
    X[r + 16 k1] (k1 < L); one exchange S[(n1, k2)]."""
    N = 16 * L
    tw = np.exp(-2j * np.pi * np.arange(N) / N)
    S = np.zeros(16 * L, complex)
    for r in range(L):
        v = np.fft.fft(V[r][:16])
        v[1:] *= tw[r * np.arange(1, 16)]
        S[r * 16 + np.arange(16)] = v
    return {r: np.fft.fft(S[np.arange(L) * 16 + r]) for r in range(16)}


def inv_16l(V, L):
    """Unnormalised inverse: thread r < 16 holds X[r + 16 k1] (k1 < L) ->
    thread r < L holds x[r + L n2] (n2 < 16)."""
    N = 16 * L
    tw = np.exp(-2j * np.pi * np.arange(N) / N)
    S = np.zeros(16 * L, complex)
    for r in range(16):
        v = np.fft.ifft(V[r][:L]) * L
        v[1:] *= np.conj(tw[r * np.arange(1, L)])
        S[np.arange(L) * 16 + r] = v
    return {r: np.fft.ifft(S[r * 16 + np.arange(16)]) * 16 for r in range(L)}


def padd_ref(X, ns, nb):
    P = np.zeros(nb, complex)
    for row in range(nb):
        if row < ns // 2:
            P[row] = X[row]
        elif row > nb - ns // 2:
            P[row] = X[row - (nb - ns)]
    return P


def unpadd_ref(X, nb, ns):
    P = np.zeros(ns, complex)
    for row in range(ns):
        if row < ns // 2:
            P[row] = X[row]
        elif row > ns // 2:
            P[row] = X[row + (nb - ns)]
    return P


@pytest.mark.parametrize("A", [8, 16])
@pytest.mark.parametrize("fwd", [True, False])
def test_pad(A, fwd):
    B = 3 * A // 2
    ns, nb = 16 * A, 16 * B
    rng = np.random.default_rng(A + 2 * fwd)
    x = rng.standard_normal(ns) + 1j * rng.standard_normal(ns)
    if fwd:  # forward transform of the input first (DIR_BOTH)
        X = fwd_16l({r: x[r + A * np.arange(16)] for r in range(A)}, A)
    else:  # the input is the spectrum (DIR_INV)
        X = {r: x[r + 16 * np.arange(A)] for r in range(16)}
    V = {}
    for r in range(16):
        v = np.zeros(max(16, B), complex)
        v[:A] = X[r][:A]
        v[A // 2 + B - A:B] = v[A // 2:A]  # small row r + 16 i -> big row r + 16 (i + B - A)
        v[A // 2:B - A // 2] = 0
        if r == 0:
            v[B - A // 2] = 0  # small Nyquist row dropped
        V[r] = v
    out = inv_16l(V, B)
    y = np.zeros(nb, complex)
    for r in range(B):
        y[r + B * np.arange(16)] = out[r]
    ref = np.fft.ifft(padd_ref(np.fft.fft(x) if fwd else x, ns, nb)) * nb
    assert np.abs(y - ref).max() <= 1e-11 * np.abs(ref).max()


@pytest.mark.parametrize("A", [8, 16])
def test_unpad(A):
    B = 3 * A // 2
    ns, nb = 16 * A, 16 * B
    rng = np.random.default_rng(100 + A)
    x = rng.standard_normal(nb) + 1j * rng.standard_normal(nb)
    X = fwd_16l({r: x[r + B * np.arange(16)] for r in range(B)}, B)
    V = {}
    for r in range(16):
        v = X[r].copy()
        v[A // 2:A] = v[A // 2 + B - A:B]  # big row r + 16 (i + B - A) -> small row r + 16 i
        if r == 0:
            v[A // 2] = 0
        V[r] = v
    out = inv_16l(V, A)
    y = np.zeros(ns, complex)
    for r in range(A):
        y[r + A * np.arange(16)] = out[r]
    ref = np.fft.ifft(unpadd_ref(np.fft.fft(x), nb, ns)) * ns
    assert np.abs(y - ref).max() <= 1e-11 * np.abs(ref).max()
