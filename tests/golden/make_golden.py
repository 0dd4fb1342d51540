"""Generate tests/golden/*.npz: an independent numpy restatement of SPECTER's hot path.

This is a second, vectorised restatement of the reference algorithm (numpy.fft
for the transforms, matrix products for the FC-Gram continuation).  Its outputs
on small seeded inputs are committed as fixtures; tests/test_oracle_golden.py
checks the C oracle against them, so the two restatements pin each other.

Reference routines restated (file:line in specter-cfd/SPECTER):
  fftp3d_real_to_complex / complex_to_real      src/fftp/fftp.fpp:388-425, 789-821
  FC-Gram continuation                          src/fftp/fftp.fpp:755-773
  dir = A . Q^T                                 src/fftp/fcgram_mod.f90:250-252
  derivk / laplak / gradre / fc_filter          src/pseudo/pseudospec_hd.f90:28-127, 209-319, 1082-1115
  advect                                        src/pseudo/pseudospec_phd.f90:23-113
  sol_project / poisson / laplace_z (Neumann)   src/boundary/boundary_mod.fpp:197-678
  v_imposebc_and_project / noslip_z             src/boundary/vboundary.f90:67-211
  s_imposebc / s_constant_z                     src/boundary/sboundary.f90:67-165
  hd / bouss stage bodies                       src/include/hd/hd_rkstep2.f90, src/include/bouss/bouss_rkstep2.f90
  energy (kin=1, kin=0 quirk), divergence       src/pseudo/pseudospec_hd.f90:405-635, 1118-1235

Run:  python tests/golden/make_golden.py     (writes tests/golden/golden_small.npz)
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = os.path.join(os.path.dirname(os.path.dirname(HERE)), "specter_gb300", "tables")


class NpGrid:
    def __init__(self, nx, ny, nz, cz=25, oz=5, Lx=1.0, Ly=1.0, Lz=1.0):
        self.nx, self.ny, self.nz, self.cz, self.oz = nx, ny, nz, cz, oz
        self.nxh, self.nzp = nx // 2 + 1, nz - cz
        self.Lz = Lz
        A = np.fromfile(os.path.join(TABLES, f"A{cz}-{oz}.dat"), "<f8").reshape(oz, cz).T
        Q = np.fromfile(os.path.join(TABLES, f"Q{oz}.dat"), "<f8").reshape(oz, oz).T
        self.dir = A @ Q.T
        self.Dkx, self.Dky = 1.0 / Lx, 1.0 / Ly
        dz = Lz / (nz - cz - 1)
        self.Dkz = 2 * np.pi / (dz * nz)
        self.z = dz * np.arange(nz)
        idx = lambda n: np.concatenate([np.arange(n // 2), np.arange(n // 2) - n // 2]).astype(float)
        self.kx = (idx(nx) * self.Dkx)[: self.nxh]
        self.ky = idx(ny) * self.Dky
        self.kz = idx(nz) * self.Dkz
        self.KX = self.kx[:, None, None]
        self.KY = self.ky[None, :, None]
        self.KZ = self.kz[None, None, :]
        self.kk2 = self.KX ** 2 + self.KY ** 2 + self.KZ ** 2
        self.khom = np.sqrt(self.kx[:, None] ** 2 + self.ky[None, :] ** 2)

    # fftp --------------------------------------------------------------------
    def cont(self, f):
        n, C, d = self.nz, self.cz, self.oz
        T = f[..., n - C - d:n - C]
        B = f[..., d - 1::-1][..., :d]
        f = f.copy()
        f[..., n - C:] = T @ self.dir.T + B @ self.dir[::-1].T
        return f

    def r2c_z(self, c):
        return np.fft.fft(self.cont(c), axis=-1)

    def c2r_z(self, c):
        return np.fft.ifft(c, axis=-1) * self.nz

    def r2c_xy(self, r):  # r (z, y, x) -> (kx, ky, z)
        return np.fft.rfft2(r, axes=(1, 2)).transpose(2, 1, 0).copy()

    def c2r_xy(self, c):
        return np.fft.irfft2(c.transpose(2, 1, 0), s=(self.ny, self.nx), axes=(1, 2)) * (self.nx * self.ny)

    def r2c(self, r):
        return self.r2c_z(self.r2c_xy(r))

    def c2r(self, c):
        return self.c2r_xy(self.c2r_z(c))

    # pseudo ------------------------------------------------------------------
    def derivk(self, a, d):
        k = (self.KX, self.KY, self.KZ)[d - 1]
        return 1j * k * a

    def curlk(self, a, b, d):
        if d == 1:
            return self.derivk(b, 2) - self.derivk(a, 3)
        if d == 2:
            return self.derivk(a, 3) - self.derivk(b, 1)
        return self.derivk(b, 1) - self.derivk(a, 2)

    def gradre(self, a, b, c):
        tmp = 1.0 / (float(self.nx) * self.ny * self.nz) ** 2
        comp = (a, b, c)
        acc = [0.0, 0.0, 0.0]
        for d in (1, 2, 3):
            r1 = self.c2r(comp[d - 1])
            for i, v in enumerate(comp):
                acc[i] = acc[i] + r1 * self.c2r(self.derivk(v, d))
        return [self.r2c(x * tmp) for x in acc]

    def advect(self, a, b, c, th):
        tmp = 1.0 / (float(self.nx) * self.ny * self.nz) ** 2
        acc = 0.0
        for d, v in zip((1, 2, 3), (a, b, c)):
            acc = acc + self.c2r(v) * self.c2r(self.derivk(th, d))
        return self.r2c(acc * tmp)

    def fc_filter(self, a):
        al = 16 * np.log(10.0)
        f = lambda k, n, dk: np.exp(-al * (2 * k / n / dk) ** 100)
        return a * f(self.KX, self.nx, self.Dkx) * f(self.KY, self.ny, self.Dky) * f(self.KZ, self.nz, self.Dkz)

    def _mean(self, r):
        w = np.full(self.nxh, 2.0)
        w[0] = 1.0
        tmp = 1.0 / (float(self.nx) * self.ny * self.nz) ** 2 / (self.nz - self.cz)
        return float(np.sum(w[:, None, None] * r[:, :, : self.nzp]) * tmp)

    def energy(self, a, b, c, kin):
        if kin == 1:
            fs = (a, b, c)
        else:  # reference quirk: y-curl twice, no z-curl
            fs = (self.curlk(b, c, 1), self.curlk(a, c, 2), self.curlk(a, c, 2))
        return self._mean(sum(np.abs(self.c2r_z(f)) ** 2 for f in fs))

    def divergence(self, a, b, c):
        return self._mean(np.abs(self.c2r_z(self.derivk(a, 1) + self.derivk(b, 2) + self.derivk(c, 3))) ** 2)

    # boundary -------------------------------------------------------------
    def sol_project(self, a, b, c):
        with np.errstate(invalid="ignore", divide="ignore"):
            d = -1j * (self.KX * a + self.KY * b + self.KZ * c) / self.kk2
        d[0, 0, 0] = 0
        a = a - 1j * self.KX * d
        b = b - 1j * self.KY * d
        c = c - 1j * self.KZ * d
        C1 = self.c2r_z(c / self.nz)
        b1, b2 = C1[:, :, 0], C1[:, :, self.nzp - 1]
        kh, Lz = self.khom, self.Lz
        with np.errstate(invalid="ignore", divide="ignore"):
            e = np.exp(-kh * Lz)
            tmp = 1.0 / (kh * (1 - np.exp(-2 * kh * Lz)))
            c1 = (b2 - b1 * e) * tmp
            c2 = (-b1 + b2 * e) * tmp
        c1[0, 0], c2[0, 0] = b1[0, 0], 0.0
        Z = self.z[None, None, :]
        K = kh[:, :, None]
        e1, e2 = np.exp(K * (Z - Lz)), np.exp(-K * Z)
        A = c1[:, :, None] * e1 + c2[:, :, None] * e2
        Bp = K * (c1[:, :, None] * e1 - c2[:, :, None] * e2)
        A[0, 0, :] = c1[0, 0].real * self.z + c2[0, 0].real
        Bp[0, 0, :] = c1[0, 0].real
        pr = self.c2r_z(d) / self.nz + A
        A, Bp = self.r2c_z(A), self.r2c_z(Bp)
        return a - 1j * self.KX * A, b - 1j * self.KY * A, c - Bp, pr

    def v_imposebc_and_project(self, vx, vy, vz, pr, o, ord, vzsta=(0.0, 0.0), vzend=(0.0, 0.0)):
        vx, vy = self.c2r_z(vx), self.c2r_z(vy)
        vx[:, :, : self.nzp] /= self.nz
        vy[:, :, : self.nzp] /= self.nz
        tmp = 1.0 / o if o == ord else (o + 1) / o
        for ind, vb in ((0, vzsta), (self.nzp - 1, vzend)):
            vx[:, :, ind] = 1j * self.kx[:, None] * pr[:, :, ind] * tmp
            vy[:, :, ind] = 1j * self.ky[None, :] * pr[:, :, ind] * tmp
            vx[0, 0, ind] = self.nx * self.ny * vb[0]
            vy[0, 0, ind] = self.nx * self.ny * vb[1]
        return self.sol_project(self.r2c_z(vx), self.r2c_z(vy), vz)

    def s_imposebc(self, th):
        t = self.c2r_z(th)
        t[:, :, : self.nzp] /= self.nz
        t[:, :, 0] = 0
        t[:, :, self.nzp - 1] = 0
        return self.r2c_z(t)

    # stages -------------------------------------------------------------------
    def hd_stage(self, p, o, v, pr, Cs):
        rmp = 1.0 / o
        N = [self.fc_filter(x) for x in self.gradre(*v)]
        v = [Cc + p["dt"] * (p["nu"] * (-self.kk2 * x) - n) * rmp for x, n, Cc in zip(v, N, Cs)]
        vx, vy, vz, pr = self.v_imposebc_and_project(*v, pr, o, p["ord"])
        return [vx, vy, vz], pr

    def bouss_stage(self, p, o, v, th, pr, Cs, C7):
        rmp = 1.0 / o
        N = self.gradre(*v)
        N8 = self.advect(*v, th)
        N[2] = N[2] - p["xmom"] * th
        N8 = N8 - p["xtemp"] * v[2]
        N = [self.fc_filter(x) for x in N]
        N8 = self.fc_filter(N8)
        vn = [Cc + p["dt"] * (p["nu"] * (-self.kk2 * x) - n) * rmp for x, n, Cc in zip(v, N, Cs)]
        th = C7 + p["dt"] * (p["kappa"] * (-self.kk2 * th) - N8) * rmp
        vx, vy, vz, pr = self.v_imposebc_and_project(*vn, pr, o, p["ord"])
        th = self.fc_filter(self.s_imposebc(th))
        th = self.r2c(self.c2r(th) / self.nx / self.ny / self.nz)
        return [vx, vy, vz], th, pr

    def run(self, p, nsteps, v, pr, th=None):
        for _ in range(nsteps):
            Cs = [x.copy() for x in v]
            C7 = th.copy() if th is not None else None
            for o in range(p["ord"], 0, -1):
                if th is None:
                    v, pr = self.hd_stage(p, o, v, pr, Cs)
                else:
                    v, th, pr = self.bouss_stage(p, o, v, th, pr, Cs, C7)
        return v, pr, th


def smooth_field(g, rng, kmax=3):
    """A seeded smooth real field on the physical rows (zeros in the continuation rows)."""
    x = 2 * np.pi * np.arange(g.nx) / g.nx
    y = 2 * np.pi * np.arange(g.ny) / g.ny
    Z, Y, X = np.meshgrid(g.z, y, x, indexing="ij")
    r = np.zeros_like(X)
    for _ in range(6):
        kx, ky = rng.integers(-kmax, kmax + 1, 2)
        kz = rng.uniform(0.5, 3.0)
        r += rng.standard_normal() * np.cos(kx * X + ky * Y + kz * Z + rng.uniform(0, 2 * np.pi))
    r[g.nzp:] = 0.0
    return r


def main():
    rng = np.random.default_rng(20261203)
    g = NpGrid(8, 6, 11 + 25, 25, 5, 1.0, 1.0, 1.0)
    out = {}
    R = smooth_field(g, rng)
    out["r2c_in"] = R
    out["r2c_out"] = g.r2c(R)
    out["c2r_out"] = g.c2r(out["r2c_out"])
    v = [g.r2c(smooth_field(g, rng)) for _ in range(3)]
    th = g.r2c(smooth_field(g, rng))
    pr = g.c2r_z(g.r2c(smooth_field(g, rng)) * 1e-3) / g.nz
    out.update(vx=v[0], vy=v[1], vz=v[2], th=th, pr=pr)
    gx, gy, gz = g.gradre(*v)
    out.update(gradre_x=gx, gradre_y=gy, gradre_z=gz, advect=g.advect(*v, th), filt=g.fc_filter(v[0]))
    a, b, c, d = g.sol_project(*v)
    out.update(proj_a=a, proj_b=b, proj_c=c, proj_d=d)
    out["energy1"] = g.energy(*v, 1)
    out["energy0"] = g.energy(*v, 0)
    out["divergence"] = g.divergence(*v)
    p = dict(dt=1e-3, nu=1e-2, kappa=1e-2, xmom=1.0, xtemp=1.0, ord=2)
    (hx, hy, hz), hpr, _ = g.run(p, 1, v, pr)
    out.update(hd_vx=hx, hd_vy=hy, hd_vz=hz, hd_pr=hpr)
    (bx, by, bz), bpr, bth = g.run(p, 1, v, pr, th)
    out.update(bo_vx=bx, bo_vy=by, bo_vz=bz, bo_th=bth, bo_pr=bpr)
    out["grid"] = np.array([g.nx, g.ny, g.nz, g.cz, g.oz], dtype=np.int64)
    out["box"] = np.array([1.0, 1.0, 1.0])
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)
    print("wrote", os.path.join(HERE, "golden_small.npz"))


if __name__ == "__main__":
    main()
