"""The algorithms of the float-float z engines, restated in numpy (complex128) and checked against
numpy.fft on the CPU.

ffblue.cuh: a 538-point z column by Bluestein over L = 1080 = 8 x 15 x 9 in three register steps
(index maps n = n3 + 9 n2 + 135 n1, k = k1 + 8 k2 + 120 k3; twiddles w_120^(n2 k1) and
w_1080^(n3 (k1 + 8 k2)); frequency k at row k3 + 9 k2 + 135 k1), the inverse by the transposed
sequence, the forward transform as conj(inverse(conj x)), and the register DFTs in the forms the
kernels use (DFT_5 with (c1 + c2)/2 = -1/4 and (c1 - c2)/2 = sqrt(5)/4, DFT_9 as 3 x 3 with
twiddles, DFT_15 prime-factor 5 x 3).

ffzoom.cuh: a wall round trip as a window correction -- the spectrum plus the forward transform of
the change on the 35 rows around the walls -- with the window values and the window transform as
chirp-z convolutions of length 576 = 8 x 8 x 9.
"""
import numpy as np
import pytest

RNG = np.random.default_rng(2026)


def w(t, n):
    return np.exp(-2j * np.pi * np.asarray(t) / n)


# ---- register DFTs (the kernels' forms) ---------------------------------------------------------
def dft3(a0, a1, a2, s):
    t, d = a1 + a2, a1 - a2
    m = a0 - 0.5 * t
    r = 1j * s * (np.sqrt(3) / 2) * d
    return a0 + t, m + r, m - r


def dft5(a, s):
    a0, a1, a2, a3, a4 = a
    t1, t2, t3, t4 = a1 + a4, a2 + a3, a1 - a4, a2 - a3
    u, v = t1 + t2, t1 - t2
    b = a0 - 0.25 * u
    dv = (np.sqrt(5) / 4) * v
    m1, m2 = b + dv, b - dv
    s51, s52 = np.sin(2 * np.pi / 5), np.sin(4 * np.pi / 5)
    n1 = 1j * s * (s51 * t3 + s52 * t4)
    n2 = 1j * s * (s52 * t3 - s51 * t4)
    return [a0 + u, m1 + n1, m2 + n2, m2 - n2, m1 - n1]


def dft9(a, s):
    a = list(a)
    for q in range(3):
        a[q], a[3 + q], a[6 + q] = dft3(a[q], a[3 + q], a[6 + q], s)
    w9 = lambda m: np.exp(s * 2j * np.pi * m / 9)
    a[4] *= w9(1)
    a[7] *= w9(2)
    a[5] *= w9(2)
    a[8] *= w9(4)
    y = [None] * 9
    for r in range(3):
        b0, b1, b2 = dft3(a[3 * r], a[3 * r + 1], a[3 * r + 2], s)
        y[r], y[r + 3], y[r + 6] = b0, b1, b2
    return y


def dft15(a, s):
    y = [[a[(3 * n1 + 5 * n2) % 15] for n2 in range(3)] for n1 in range(5)]
    for n1 in range(5):
        y[n1] = list(dft3(*y[n1], s))
    out = [None] * 15
    for k2 in range(3):
        col = dft5([y[n1][k2] for n1 in range(5)], s)
        for k1 in range(5):
            out[(6 * k1 + 10 * k2) % 15] = col[k1]
    return out


def dft8(a, s):
    e = [a[0], a[2], a[4], a[6]]
    o = [a[1], a[3], a[5], a[7]]

    def dft4(x):
        t0, t1, t2, t3 = x[0] + x[2], x[0] - x[2], x[1] + x[3], 1j * s * (x[1] - x[3])
        return [t0 + t2, t1 + t3, t0 - t2, t1 - t3]

    e, o = dft4(e), dft4(o)
    h = np.sqrt(0.5)
    o = [o[0], h * (o[1] + 1j * s * o[1]), 1j * s * o[2], h * (1j * s * o[3] - o[3])]
    return [e[k] + o[k] for k in range(4)] + [e[k] - o[k] for k in range(4)]


@pytest.mark.parametrize("s", [-1, 1])
def test_register_dfts(s):
    for n, f in ((3, lambda a: dft3(*a, s)), (5, lambda a: dft5(a, s)), (8, lambda a: dft8(a, s)),
                 (9, lambda a: dft9(a, s)), (15, lambda a: dft15(a, s))):
        x = RNG.standard_normal(n) + 1j * RNG.standard_normal(n)
        ref = np.fft.fft(x) if s < 0 else np.fft.ifft(x) * n
        got = np.array(f(list(x)))
        assert np.allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max()), n


# ---- three-step transforms ----------------------------------------------------------------------
def three_step_forward(x, L1, L2, L3, dfts):
    """Forward DFT of length L1 L2 L3 in the kernels' three steps; returns the buffer with
    frequency k1 + L1 k2 + L1 L2 k3 at row k3 + L3 k2 + L2 L3 k1."""
    M, J, L = L2 * L3, L1 * L2, L1 * L2 * L3
    X = np.array(x, complex)
    for np_ in range(M):                                   # step A
        n2 = np_ // L3
        a = dfts[L1]([X[np_ + M * n1] for n1 in range(L1)], -1)
        for k1 in range(L1):
            X[np_ + M * k1] = a[k1] * w(n2 * k1, J)
    for j in range(L1 * L3):                               # step B
        k1, n3 = divmod(j, L3)
        base = n3 + M * k1
        b = dfts[L2]([X[base + L3 * n2] for n2 in range(L2)], -1)
        for k2 in range(L2):
            X[base + L3 * k2] = b[k2] * w(n3 * (k1 + L1 * k2), L)
    for j in range(J):                                     # step C
        k1, k2 = divmod(j, L2)
        base = L3 * k2 + M * k1
        X[base:base + L3] = dfts[L3](list(X[base:base + L3]), -1)
    return X


def three_step_inverse(X, L1, L2, L3, dfts):
    """Unnormalised inverse from the permuted layout back to natural order (steps C', B', A')."""
    M, J, L = L2 * L3, L1 * L2, L1 * L2 * L3
    X = np.array(X, complex)
    for j in range(J):
        k1, k2 = divmod(j, L2)
        base = L3 * k2 + M * k1
        d = dfts[L3](list(X[base:base + L3]), +1)
        for m3 in range(L3):
            X[base + m3] = d[m3] * np.conj(w(m3 * (k1 + L1 * k2), L))
    for j in range(L1 * L3):
        k1, m3 = divmod(j, L3)
        base = m3 + M * k1
        b = dfts[L2]([X[base + L3 * k2] for k2 in range(L2)], +1)
        for m2 in range(L2):
            X[base + L3 * m2] = b[m2] * np.conj(w(m2 * k1, J))
    out = np.empty(L, complex)
    for mp in range(M):
        a = dfts[L1]([X[mp + M * k1] for k1 in range(L1)], +1)
        for m1 in range(L1):
            out[mp + M * m1] = a[m1]
    return out


DFTS = {8: dft8, 9: dft9, 15: dft15}


@pytest.mark.parametrize("split", [(8, 15, 9), (8, 8, 9)], ids=["1080", "576"])
def test_three_step_index_maps(split):
    L1, L2, L3 = split
    L = L1 * L2 * L3
    x = RNG.standard_normal(L) + 1j * RNG.standard_normal(L)
    X = three_step_forward(x, L1, L2, L3, DFTS)
    F = np.fft.fft(x)
    k = np.arange(L)
    k1, rest = k % L1, k // L1
    k2, k3 = rest % L2, rest // L2
    rows = k3 + L3 * k2 + L2 * L3 * k1
    assert np.allclose(X[rows], F, atol=1e-11 * np.abs(F).max())
    back = three_step_inverse(X, L1, L2, L3, DFTS)
    assert np.allclose(back / L, x, atol=1e-12)


def test_bluestein_1080_with_conjugation():
    """n = 538 over L = 1080: the inverse transform's chirp and filter only, the forward transform
    as conj(inverse(conj x)); the filter applied in the permuted order of the third step."""
    n, L = 538, 1080
    c = np.exp(1j * np.pi * (np.arange(n) ** 2 % (2 * n)) / n)        # exp(+i pi k^2 / n)
    b = np.zeros(L, complex)
    b[:n] = np.conj(c)
    b[L - n + 1:] = np.conj(c[1:])[::-1]
    H = np.fft.fft(b) / L

    def inverse(x):  # sum_k x_k exp(+2 pi i j k / n)
        a = np.zeros(L, complex)
        a[:n] = x * c
        return (np.fft.ifft(np.fft.fft(a) * H) * L)[:n] * c

    x = RNG.standard_normal(n) + 1j * RNG.standard_normal(n)
    assert np.allclose(inverse(x), np.fft.ifft(x) * n, atol=1e-10)
    assert np.allclose(np.conj(inverse(np.conj(x))), np.fft.fft(x), atol=1e-10)
    # the kernels' half-zero first step: the input rows n .. L/2 - 1 and the upper half are zero
    assert n <= L // 2


# ---- window corrections -------------------------------------------------------------------------
N, C, D = 538, 25, 5
NZP = N - C
J0, WIN, LW = NZP - D, C + 2 * D, 576


def chirp(k):
    k = np.asarray(k) % N
    return np.exp(1j * np.pi * (k * k % (2 * N)) / N)


def window_values(X):
    """(1): rows j0 + m (mod n), m < 35, of the unnormalised inverse transform, as a length-576
    cyclic convolution of X_k c_k with g[s] = conj(c_{j0+s})."""
    a = np.zeros(LW, complex)
    a[:N] = X * chirp(np.arange(N))
    g = np.zeros(LW, complex)
    for s in range(-(N - 1), WIN):
        g[s % LW] = np.conj(chirp(J0 + s))
    y = np.fft.ifft(np.fft.fft(a) * np.fft.fft(g))[:WIN]
    return y * chirp(J0 + np.arange(WIN))


def window_transform(dv):
    """(2): sum_p dv_p exp(-2 pi i (j0 + p) k / n), k < n, as a length-576 cyclic convolution of
    dv_p conj(c_{j0+p}) with h[s] = c_{s-j0}."""
    a = np.zeros(LW, complex)
    a[:WIN] = dv * np.conj(chirp(J0 + np.arange(WIN)))
    h = np.zeros(LW, complex)
    for s in range(-(WIN - 1), N):
        h[s % LW] = chirp(s - J0)
    z = np.fft.ifft(np.fft.fft(a) * np.fft.fft(h))[:N]
    return z * np.conj(chirp(np.arange(N)))


def test_window_chirp_z():
    assert N + WIN - 1 <= LW
    X = RNG.standard_normal(N) + 1j * RNG.standard_normal(N)
    rows = (J0 + np.arange(WIN)) % N
    assert np.allclose(window_values(X), (np.fft.ifft(X) * N)[rows], atol=1e-10)
    dv = RNG.standard_normal(WIN) + 1j * RNG.standard_normal(WIN)
    full = np.zeros(N, complex)
    full[rows] = dv
    assert np.allclose(window_transform(dv), np.fft.fft(full), atol=1e-10)


def test_round_trip_as_window_correction():
    """A wall round trip (inverse, new wall rows, continuation rebuilt from the 2d wall-adjacent
    rows, forward) equals the spectrum plus the forward transform of the window's change."""
    dirm = RNG.standard_normal((C, D)) * 10      # any continuation operator: the identity is linear
    dirb = RNG.standard_normal((C, D)) * 10
    X = RNG.standard_normal(N) + 1j * RNG.standard_normal(N)
    walls = (0.3 + 0.1j, -0.2j)

    def modify(u):
        u = u.copy()
        u[0], u[NZP - 1] = walls
        top, bot = u[NZP - D:NZP], u[D - 1::-1]
        u[NZP:] = dirm @ top + dirb @ bot
        return u

    plain = np.fft.fft(modify(np.fft.ifft(X)))
    rows = (J0 + np.arange(WIN)) % N
    u = window_values(X) / N
    full = np.fft.ifft(X)
    assert np.allclose(u, full[rows], atol=1e-12)
    new = modify(full)[rows]
    dv = new - u
    assert np.count_nonzero(np.abs(dv) > 1e-13) <= C + 2     # walls and continuation rows only
    got = X + window_transform(dv)
    assert np.allclose(got, plain, atol=1e-9 * np.abs(plain).max())
