"""Seeded initial conditions: solenoidal, zero at the walls, requested amplitude (CPU)."""
import numpy as np

from specter_gb300.initial import channel_velocity, convection_theta


class _Plan:
    def __init__(self, nx, ny, nzp, cz, Lz):
        self.nx, self.ny, self.nzp, self.nz = nx, ny, nzp, nzp + cz
        self.lengths = (1.0, 1.0, Lz)
        dz = Lz / (nzp - 1)
        self.z = [dz * k for k in range(self.nz)]


def test_channel_ic():
    p = _Plan(32, 32, 65, 25, 2.0)
    ux, uy, uz = channel_velocity(p, seed=1, amp=0.05, kmax=8)
    z = np.asarray(p.z[:65])
    for u in (ux, uy, uz):
        assert np.all(u[65:] == 0)
        assert np.abs(u[0]).max() == 0 and np.abs(u[64]).max() < 1e-14
    pert = [ux[:65] - (1 - (z[:, None, None] - 1) ** 2), uy[:65], uz[:65]]
    assert abs(np.sqrt(np.mean(sum(a ** 2 for a in pert))) - 0.05) < 1e-12
    # divergence-free up to the O(dz^2) error of the finite-difference z derivative used here
    k = np.fft.fftfreq(32, 1 / 32)
    dudx = np.fft.ifft(1j * k[None, None, :] * np.fft.fft(ux[:65], axis=2), axis=2).real
    dvdy = np.fft.ifft(1j * k[None, :, None] * np.fft.fft(uy[:65], axis=1), axis=1).real
    dwdz = np.gradient(uz[:65], z[1] - z[0], axis=0, edge_order=2)
    assert np.sqrt(np.mean((dudx + dvdy + dwdz) ** 2)) < 0.02 * np.sqrt(np.mean(dudx ** 2))
    # seeded: same seed, same field
    assert np.array_equal(channel_velocity(p, seed=1)[2], uz)


def test_convection_ic():
    p = _Plan(16, 16, 33, 25, 1.0)
    th = convection_theta(p, seed=3, amp=1e-3)
    assert np.all(th[0] == 0) and np.abs(th[32]).max() < 1e-18 and np.all(th[33:] == 0)
    assert np.abs(th).max() <= 1e-3 * 0.25 + 1e-15
