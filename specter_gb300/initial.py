"""Seeded initial conditions of the benchmark configurations (physical space, host).

The reference's IC hooks are user code INCLUDEd by the driver (src/initialv.f90,
src/initials.f90); the channel and convection cases here define their own fields:

* channel (HD): u = (U(z), 0, 0) + u',  U = 1 - (z/h - 1)^2 with h = Lz/2 (Poiseuille,
  U = 0 at both walls), and u' = curl(env(z) * A) with env = z^2 (Lz - z)^2 and
  A = (A1, A2, A3) a sum of random-phase modes cos(kx x + ky y + phi) * cos(kz z + psi),
  kx, ky integers, kz = pi*m/Lz (m >= 1), 1 <= |k| <= kmax.  u' is solenoidal and vanishes
  with zero slope at the walls (env and env' are zero there).  u' is scaled to rms = amp
  over the physical grid.
* convection (BOUSS): theta' = 1e-3 * xi * z (Lz - z) with xi ~ U(-1, 1) white noise,
  v = 0.  theta' is the deviation from the linear conduction profile (theta' = 0 on both
  walls); the mean gradient enters through the heat-current term -xtemp*vz of the scalar
  equation (bouss_rkstep2.f90:15) and buoyancy through -xmom*theta (:14).

Random numbers: numpy PCG64 seeded with the given 64-bit seed.  Fields are returned in the
reference's physical layout (nz, ny, nx) with zeros on the Cz continuation rows.
"""
from __future__ import annotations

import numpy as np


def _grid(plan):
    nx, ny, nzp = plan.nx, plan.ny, plan.nzp
    Lx, Ly, Lz = plan.lengths
    x = 2 * np.pi * Lx * np.arange(nx) / nx
    y = 2 * np.pi * Ly * np.arange(ny) / ny
    z = np.asarray(plan.z[:nzp])
    return x, y, z, Lx, Ly, Lz


def channel_velocity(plan, seed=1234, amp=0.05, kmax=8):
    """Poiseuille + solenoidal perturbation; returns (ux, uy, uz) real arrays (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    x, y, z, Lx, Ly, Lz = _grid(plan)
    nx, ny, nzp = plan.nx, plan.ny, plan.nzp
    env = z ** 2 * (Lz - z) ** 2
    denv = 2 * z * (Lz - z) ** 2 - 2 * z ** 2 * (Lz - z)
    # per z-mode m: 2-D random-phase spectra for A1, A2, A3 restricted to |k| <= kmax
    kxv = np.fft.fftfreq(nx, d=1.0 / nx) / Lx
    kyv = np.fft.fftfreq(ny, d=1.0 / ny) / Ly
    KX, KY = np.meshgrid(kxv, kyv, indexing="xy")  # (ny, nx)
    mmax = int(np.floor(kmax * Lz / np.pi))
    comps = {n: np.zeros((nzp, ny, nx)) for n in ("A1", "A2", "A3", "dzA1", "dzA2", "dxA2", "dxA3", "dyA1", "dyA3")}
    for m in range(1, max(mmax, 1) + 1):
        kz = np.pi * m / Lz
        mask = (KX ** 2 + KY ** 2 + kz ** 2) <= kmax ** 2
        if not mask.any():
            continue
        psi = rng.uniform(0, 2 * np.pi)
        cz, sz = np.cos(kz * z + psi), -kz * np.sin(kz * z + psi)
        for name in ("A1", "A2", "A3"):
            spec = np.zeros((ny, nx), complex)
            nmode = int(mask.sum())
            spec[mask] = (rng.standard_normal(nmode) + 1j * rng.standard_normal(nmode))
            f = np.fft.ifft2(spec).real
            comps[name] += f[None] * cz[:, None, None]
            if name in ("A1", "A2"):
                comps["dz" + name] += f[None] * sz[:, None, None]
            dx = np.fft.ifft2(1j * KX * spec).real
            dy = np.fft.ifft2(1j * KY * spec).real
            if name in ("A2", "A3"):
                comps["dx" + name] += dx[None] * cz[:, None, None]
            if name in ("A1", "A3"):
                comps["dy" + name] += dy[None] * cz[:, None, None]
    E, D = env[:, None, None], denv[:, None, None]
    c = comps
    ux = E * (c["dyA3"] - c["dzA2"]) - D * c["A2"]
    uy = E * (c["dzA1"] - c["dxA3"]) + D * c["A1"]
    uz = E * (c["dxA2"] - c["dyA1"])
    rms = np.sqrt(np.mean(ux ** 2 + uy ** 2 + uz ** 2))
    s = amp / rms if rms > 0 else 0.0
    h = Lz / 2
    U = 1.0 - (z / h - 1.0) ** 2
    out = []
    for k, u in enumerate((ux, uy, uz)):
        full = np.zeros((plan.nz, ny, nx))
        full[:nzp] = u * s + (U[:, None, None] if k == 0 else 0.0)
        out.append(full)
    return out


def convection_theta(plan, seed=1234, amp=1e-3):
    """theta' = amp * xi * z (Lz - z), xi ~ U(-1, 1); returns a real array (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    x, y, z, Lx, Ly, Lz = _grid(plan)
    xi = rng.uniform(-1.0, 1.0, size=(plan.nzp, plan.ny, plan.nx))
    full = np.zeros((plan.nz, plan.ny, plan.nx))
    full[: plan.nzp] = amp * xi * (z * (Lz - z))[:, None, None]
    return full


def to_spectral(plan, real_fields):
    """r2c of physical fields on the GPU; returns Field handles."""
    from . import api
    out = []
    for r in real_fields:
        fr = plan.field(api.REAL, data=r.astype(plan.rdtype))
        fc = plan.field(api.COMPLEX)
        api.fftp3d_real_to_complex(plan, fr, fc)
        out.append(fc)
    return out
