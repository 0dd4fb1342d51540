"""Conditioning of the FC-Gram continuation (CPU): how much FP32 input rounding costs.

dir = A.Q^T (fcgram_mod.f90:250-252) has row sums of |dir| up to 9.5e3 for C = 25, d = 5, so
the continuation amplifies any error in the d wall-adjacent points.  This fixes the accuracy
floor of any FP32 form of the FC-Gram transform (the reference's single-precision build
included): FP32 storage of a smooth column alone already costs ~1e-5 relative in its spectrum.
"""
import os

import numpy as np

TABLES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "specter_gb300", "tables")


def _dir():
    A = np.fromfile(os.path.join(TABLES, "A25-5.dat"), "<f8").reshape(5, 25).T
    Q = np.fromfile(os.path.join(TABLES, "Q5.dat"), "<f8").reshape(5, 5).T
    return A @ Q.T


def _extend(f, D, nzp, C=25, d=5):
    g = np.zeros(nzp + C, complex)
    g[:nzp] = f
    g[nzp:] = D @ f[nzp - d:nzp] + D[::-1] @ f[d - 1::-1][:d]
    return g


def test_fp32_rounding_floor():
    D = _dir()
    assert 9.0e3 < np.abs(D).sum(1).max() < 1.0e4
    nzp = 513
    z = np.linspace(0.0, 1.0, nzp)
    rng = np.random.default_rng(0)
    errs = []
    for _ in range(8):
        f = sum(rng.standard_normal() * np.cos(rng.uniform(2, 24) * z + rng.uniform(0, 6.3)) for _ in range(6))
        f = f.astype(complex)
        f32 = f.astype(np.complex64).astype(complex)
        e64 = np.fft.fft(_extend(f, D, nzp))
        e32 = np.fft.fft(_extend(f32, D, nzp))
        errs.append(np.linalg.norm(e32 - e64) / np.linalg.norm(e64))
    # input rounding is ~3e-8; after the continuation the spectrum is off by 1e-6 .. 1e-4
    assert 1e-6 < np.median(errs) < 1e-4
