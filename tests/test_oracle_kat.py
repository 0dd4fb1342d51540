"""The reference's known-answer programs, re-run on the oracle with explicit thresholds.

The reference prints these errors without asserting (src/tests/*.f90); the
thresholds here are set from the analytic accuracy of each quantity.
"""
import numpy as np
import pytest


def _mesh(g):
    x = 2 * np.pi * g.Lx * np.arange(g.nx) / g.nx
    y = 2 * np.pi * g.Ly * np.arange(g.ny) / g.ny
    Z, Y, X = np.meshgrid(g.z, y, x, indexing="ij")
    return X, Y, Z


def test_fc_dirichlet_derivatives(channel_grid):
    """src/tests/fc_dirichlet.f90:11-89: derivatives of sin4x cos8y sin6z through r2c/derivk/c2r."""
    g = channel_grid
    X, Y, Z = _mesh(g)
    nzp = g.nz - g.cz
    c1 = g.fftp3d_real_to_complex(np.sin(4 * X) * np.cos(8 * Y) * np.sin(6 * Z))
    N = g.nx * g.ny * g.nz
    exact = {
        1: 4 * np.cos(4 * X) * np.cos(8 * Y) * np.sin(6 * Z),
        2: np.sin(4 * X) * (-8 * np.sin(8 * Y)) * np.sin(6 * Z),
        3: np.sin(4 * X) * np.cos(8 * Y) * 6 * np.cos(6 * Z),
    }
    for d, ex in exact.items():
        r = g.fftp3d_complex_to_real(g.derivk(c1, d)) / N
        err = np.abs(r[:nzp] - ex[:nzp])
        if d < 3:  # periodic directions: spectral accuracy
            assert err.max() < 1e-12
        else:  # FC-Gram (C=25, d=5) at 65 points: high-order accurate, largest at the walls
            assert err.max() < 5e-3 and err.mean() < 1e-4


def test_fft_round_trips(channel_grid):
    """src/tests/fft.f90:12-67: Z and XY transform/anti-transform round trips."""
    g = channel_grid
    X, Y, Z = _mesh(g)
    nzp = g.nz - g.cz
    r1 = np.zeros(g.rshape)
    r1[:nzp] = (np.sin(4 * X) * np.cos(8 * Y) * np.sin(6 * Z))[:nzp]
    c1 = g.fftp2d_real_to_complex_xy(r1)
    # |c(kx=4, ky=8)| = nx*ny/4 * |sin(6 z)| for the xy transform
    amp = np.abs(c1[4, 8, :nzp])
    assert np.allclose(amp, g.nx * g.ny / 4 * np.abs(np.sin(6 * g.z[:nzp])), atol=1e-9)
    c3 = g.fftp1d_real_to_complex_z(c1)
    c3 = g.fftp1d_complex_to_real_z(c3)
    assert np.abs(c1[:, :, :nzp] - c3[:, :, :nzp] / g.nz).max() < 1e-10
    r2 = g.fftp2d_complex_to_real_xy(c1)
    assert np.abs(r1[:nzp] - r2[:nzp] / g.nx / g.ny).max() < 1e-13


def test_energy_parseval(channel_grid):
    """src/tests/energy.f90:9-32: mean energy in real space vs the mixed-domain energy()."""
    g = channel_grid
    X, Y, Z = _mesh(g)
    nzp = g.nz - g.cz
    r = np.zeros(g.rshape)
    r[:nzp] = (np.sin(4 * X) * np.cos(8 * Y) * np.sin(6 * Z))[:nzp]
    tmq = np.sum(3 * r[:nzp] ** 2) / g.nx / g.ny / nzp
    c = g.fftp3d_real_to_complex(r)
    tmp = g.energy(c, c, c, 1)
    assert abs(tmq - tmp) / abs(tmq) < 1e-13


def test_poisson_projection(channel_grid):
    """src/tests/poisson.f90:15-105: divergence KAT, then sol_project with both targets."""
    g = channel_grid
    X, Y, Z = _mesh(g)
    Lz = g.Lz
    e = np.sin(4 * X) * np.cos(8 * Y) * np.exp(.4 * Z / Lz)
    c1 = g.fftp3d_real_to_complex(e)
    div_ex = np.exp(.4 * Z / Lz) * (4 * np.cos(4 * X) * np.cos(8 * Y) - 8 * np.sin(4 * X) * np.sin(8 * Y)
                                    + .4 * np.sin(4 * X) * np.cos(8 * Y) / Lz)
    c4 = g.fftp3d_real_to_complex(div_ex)
    tmp = g.energy(c4, c4, c4, 1) / 3.0
    tmq = g.divergence(c1, c1, c1)
    assert abs(tmp - tmq) / tmp < 1e-10
    # velocity target: divergence removed, normal velocity zero at the walls
    a, b, c, d = g.sol_project(c1, c1, c1, 1, 0, 0)
    assert g.divergence(a, b, c) < 1e-6 * tmp
    bot, top = g.bouncheck_z(c)
    assert bot < 1e-24 and top < 1e-24
    # potential target: potential zero at the walls
    a, b, c, d = g.sol_project(c1, c1, c1, 0, 0, 0)
    assert g.divergence(a, b, c) < 1e-6 * tmp
    pr = g.fftp1d_real_to_complex_z(d)
    bot, top = g.bouncheck_z(pr)
    assert bot < 1e-24 and top < 1e-24


def test_table_dir_matches_a_qt(channel_grid):
    """fcgram_mod.f90:250-252: dir = A . Q^T from the raw Fortran-order tables."""
    import os
    from oracle.oracle import _HERE
    tdir = os.path.join(os.path.dirname(_HERE), "specter_gb300", "tables")
    A = np.fromfile(os.path.join(tdir, "A25-5.dat"), "<f8").reshape(5, 25).T
    Q = np.fromfile(os.path.join(tdir, "Q5.dat"), "<f8").reshape(5, 5).T
    assert np.abs(Q.T @ Q - np.eye(5)).max() < 1e-14
    assert np.allclose(channel_grid.dir, A @ Q.T, rtol=0, atol=1e-12)


def test_bad_shape_rejected(oracle_mod):
    with pytest.raises(ValueError):
        oracle_mod.Grid(63, 64, 90)
    with pytest.raises(ValueError):
        oracle_mod.Grid(64, 64, 90, tdir="/nonexistent")
