"""Host-side models of the FFT planning rules, checked on the CPU:

* the per-axis four-step split lists of specter_gb300/csrc/fast.h and the Bluestein length rule
  of build_fft4_table (fast_f32.cu): every grid of the configurations and of the ensemble /
  served streams gets a compiled split on every axis;
* the Good-Thomas index maps of dft_pfa (fft4.cuh), restated with the same formulas and checked
  against numpy.fft;
* the model FFT operation count bench.py reports beside the throughput."""
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def split_lists():
    text = open(os.path.join(ROOT, "specter_gb300", "csrc", "fast.h")).read()
    out = {}
    for ax in "XYZ":
        m = re.search(r"#define SG_FAST_PAIRS_%s\(F\)(.*)" % ax, text)
        out[ax.lower()] = [(int(a), int(b)) for a, b in re.findall(r"F\((\d+),\s*(\d+)\)", m.group(1))]
    return out


def smooth235(m):
    for p in (2, 3, 5):
        while m % p == 0:
            m //= p
    return m == 1


def choose(axis, n, lists):
    """build_fft4_table: the length itself when compiled, else (z only) Bluestein over the
    smallest compiled L >= 2n - 1 with n <= L/2 and an even L1; None: generic engine."""
    pairs = {a * b: (a, b) for a, b in lists[axis]}
    if n in pairs:
        return n, pairs[n], False
    if axis != "z":
        return None
    for m in range(2 * n - 1, 4 * n + 1):
        if smooth235(m) and 2 * n <= m and m in pairs and pairs[m][0] % 2 == 0:
            return m, pairs[m], True
    return None


def test_split_lists_even_first_factor():
    for ax, pairs in split_lists().items():
        for a, b in pairs:
            assert a % 2 == 0, (ax, a, b)  # the Bluestein body halves step A / A' on L1


@pytest.mark.parametrize("nx,ny,nzp", [
    (64, 64, 65), (256, 256, 257), (512, 512, 513), (128, 128, 513),            # configurations, bench sample
    (32, 48, 33), (48, 64, 65), (64, 96, 97), (96, 32, 33),                     # ensemble draws
    (64, 128, 65), (128, 256, 129), (256, 64, 257),                             # served draws
])
def test_every_production_grid_has_a_split(nx, ny, nzp):
    lists = split_lists()
    nz = nzp + 25
    for ax, n in (("x", nx // 2), ("y", ny), ("z", nz)):
        assert choose(ax, n, lists) is not None, (ax, n)


def test_bluestein_lengths():
    lists = split_lists()
    assert choose("z", 538, lists) == (1080, (36, 30), True)
    assert choose("z", 282, lists) == (576, (24, 24), True)
    assert choose("z", 154, lists) == (320, (20, 16), True)
    assert choose("z", 122, lists) == (256, (16, 16), True)
    assert choose("z", 58, lists) == (128, (16, 8), True)
    assert choose("z", 90, lists) == (90, (10, 9), False)
    assert choose("x", 45, lists) is None  # no Bluestein on x / y: the generic engine serves it


def pfa_n1(n):
    for c in (16, 8, 4, 9, 27, 5, 3, 2):
        if c < n and n % c == 0 and math.gcd(c, n // c) == 1:
            return c
    return 0


def dft_pfa(a, sign):
    """Restatement of fft4.cuh dft_pfa (same maps), numpy for the short DFTs."""
    n = len(a)
    n1 = pfa_n1(n)
    if n1 == 0:
        return np.fft.fft(a) if sign < 0 else np.fft.ifft(a) * n
    n2 = n // n1
    e1 = n2 * pow(n2 % n1, -1, n1)
    e2 = n1 * pow(n1 % n2, -1, n2)
    y = np.array([[a[(n2 * i1 + n1 * i2) % n] for i2 in range(n2)] for i1 in range(n1)])
    y = np.array([dft_pfa(row, sign) for row in y])
    out = np.zeros(n, complex)
    for k2 in range(n2):
        col = dft_pfa(y[:, k2], sign)
        for k1 in range(n1):
            out[(e1 * k1 + e2 * k2) % n] = col[k1]
    return out


@pytest.mark.parametrize("n", [6, 10, 12, 15, 18, 20, 24, 30, 36, 40, 45])
def test_good_thomas_maps(n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert np.allclose(dft_pfa(a, -1), np.fft.fft(a), atol=1e-12)
    assert np.allclose(dft_pfa(a, +1), np.fft.ifft(a) * n, atol=1e-12)


def test_model_flops():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    f = bench.fft_flops_per_stage(bench.CFG, dict(L=1080, bluestein=True))
    nx, ny, nzp, nz = 512, 512, 513, 538
    nxh = nx // 2 + 1
    z = 23 * nxh * ny * (2 * 5 * 1080 * math.log2(1080) + 6 * (2 * nz + 1080))
    y = 16 * nxh * nzp * 5 * ny * math.log2(ny)
    x = 19 * ny * nzp * 2.5 * nx * math.log2(nx)
    assert f == pytest.approx(z + y + x)
    assert 4.5e11 < f < 5.0e11


def test_traffic_table_has_the_stage_kernels():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    t = bench.load_traffic()
    for k in ("fused_vcomp", "fused_vproj", "fused_theta", "x_nonlinear", "z_inverse", "y_inverse", "y_forward"):
        assert t.get(k, 0) > 1e9, k


def test_bluestein_half_zero_assumption():
    """The Bluestein body reads only the first L1/2 rows of each step-A column and forms only the
    first L1/2 outputs of step A' (fft4.cuh): valid when n <= L2 * (L1/2), for every z length that
    selects a Bluestein split."""
    lists = split_lists()
    seen = set()
    for n in range(8, 1200):
        c = choose("z", n, lists)
        if c is None or not c[2]:
            continue
        L, (l1, l2), _ = c
        assert 2 * n - 1 <= L and n <= l2 * (l1 // 2), (n, L, l1, l2)
        seen.add(L)
    assert {1080, 576, 320, 256, 128} <= seen


def _c2r_pre_pairs(X, H, nx):
    """kernels.cuh c2r_pre: Z_k and Z_{H-k} from X_k, X_{H-k} (one (k, H-k) pair per thread)."""
    Z = np.zeros(H, complex)
    for k in range(H // 2 + 1):
        xk, xm = X[k], X[H - k]
        if k == 0:
            xk, xm = xk.real + 0j, xm.real + 0j
        e = xk + np.conj(xm)
        w = np.exp(2j * np.pi * k / nx)
        o = (xk - np.conj(xm)) * w
        Z[k] = complex(e.real - o.imag, e.imag + o.real)
        if k != 0 and 2 * k != H:
            Z[H - k] = complex(e.real + o.imag, o.real - e.imag)
    return Z


def _r2c_post_pairs(Z, H, nx):
    """kernels.cuh r2c_post: X_k and X_{H-k} from Z_k, Z_{H-k}; k = 0 also gives X_H."""
    X = np.zeros(H + 1, complex)
    for k in range(H // 2 + 1):
        zk, zm = Z[k], np.conj(Z[(H - k) % H])
        e, d = zk + zm, zk - zm
        t = d * np.exp(-2j * np.pi * k / nx)
        X[k] = complex(0.5 * (e.real + t.imag), 0.5 * (e.imag - t.real))
        if 2 * k != H:
            X[H - k] = complex(0.5 * (e.real - t.imag), -0.5 * (e.imag + t.real))
    return X


@pytest.mark.parametrize("nx", [32, 48, 90, 256, 512])
def test_real_fft_pair_formulas(nx):
    """The paired pre-/post-processing of the x pass (a real row of nx points through a complex
    FFT of H = nx/2 points) against numpy's real transforms."""
    H = nx // 2
    rng = np.random.default_rng(nx)
    x = rng.standard_normal(nx)
    X = np.fft.rfft(x)                       # half spectrum, H + 1 values
    z = np.fft.ifft(_c2r_pre_pairs(X, H, nx)) * H  # unnormalised inverse, packed (x_2m, x_2m+1)
    assert np.allclose(z.real, np.fft.irfft(X, nx)[0::2] * nx, atol=1e-9)
    assert np.allclose(z.imag, np.fft.irfft(X, nx)[1::2] * nx, atol=1e-9)
    Zf = np.fft.fft(x[0::2] + 1j * x[1::2])  # forward FFT of the packed row
    assert np.allclose(_r2c_post_pairs(Zf, H, nx), X, atol=1e-9)
