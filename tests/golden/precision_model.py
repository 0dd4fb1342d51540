"""Which operations of a Boussinesq RK stage may run in FP32: a numpy model of the precision forms.

The FP32 rounding of the 2d wall-adjacent rows that feed an FC-Gram continuation is multiplied
by up to sum|dir| = 9.5e3 (C = 25, d = 5).  This model runs the Rayleigh-Benard configuration's z
grid (513 physical + 25 continuation points, Lz = 1, nu = kappa = 1e-4, dt = 1e-5, RK2, theta' =
1e-3 U(-1,1) z(1-z), v = 0) on a small periodic plane with the stage of bouss_rkstep2.f90
restated in numpy (the independent restatement of make_golden.py), and rounds chosen
operations to FP32 (numpy's single-precision FFTs, float32 rounding of their outputs):

  nl     the nonlinear terms (gradre, advect, their transforms and products, the filter of NL)
  upd    the RK update (rounds the updated state)
  R      the wall round trips of v_imposebc_and_project and s_imposebc (IFFT, walls,
         continuation, FFT)
  proj   sol_project
  filt   fc_filter of theta
  hack   the c2r -> /N -> r2c round trip of theta
  state  the state stored in FP32 at the end of every stage

and prints, per variant, the relative L2 error of vx, vy, vz, theta on the physical grid
against the all-FP64 run.  Every state-carrying operation in FP32 (upd, R, proj, filt, hack,
state) costs 1e-5 .. 4e-4 after 100 steps; the nonlinear term alone in FP32 costs 2.5e-7 and
its error falls to 5e-8 by step 1000 -- the split the nl_fp32 form implements.

    python tests/golden/precision_model.py NXY STEPS "VARIANT;VARIANT;..."
    e.g. python tests/golden/precision_model.py 16 100 "all32;nl=32;R=32;state=32"
"""
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from make_golden import NpGrid  # noqa: E402

C64 = np.complex64


def rnd(x, p):
    return x.astype(C64).astype(np.complex128) if p == 32 else x


class PG(NpGrid):
    def c2r_zp(self, c, p):
        if p == 32:
            return (np.fft.ifft(c.astype(C64), axis=-1) * np.float32(self.nz)).astype(np.complex128)
        return np.fft.ifft(c, axis=-1) * self.nz

    def r2c_zp(self, c, p):
        f = self.cont(rnd(c, p))  # continuation arithmetic in FP64 on inputs of precision p
        if p == 32:
            return np.fft.fft(f.astype(C64), axis=-1).astype(np.complex128)
        return np.fft.fft(f, axis=-1)

    def r2c_xyp(self, r, p):
        if p == 32:
            return np.fft.rfft2(r.astype(np.float32), axes=(1, 2)).transpose(2, 1, 0).astype(np.complex128)
        return self.r2c_xy(r)

    def c2r_xyp(self, c, p):
        if p == 32:
            return (np.fft.irfft2(c.transpose(2, 1, 0).astype(C64), s=(self.ny, self.nx), axes=(1, 2))
                    * np.float32(self.nx * self.ny)).astype(np.float64)
        return self.c2r_xy(c)

    def c2rp(self, c, p):
        return self.c2r_xyp(self.c2r_zp(c, p), p)

    def r2cp(self, r, p):
        return self.r2c_zp(self.r2c_xyp(r, p), p)

    def gradre_p(self, a, b, c, p):
        tmp = 1.0 / (float(self.nx) * self.ny * self.nz) ** 2
        comp = (a, b, c)
        acc = [0.0, 0.0, 0.0]
        for d in (1, 2, 3):
            r1 = self.c2rp(comp[d - 1], p)
            for i, v in enumerate(comp):
                acc[i] = acc[i] + r1 * self.c2rp(rnd(self.derivk(v, d), p), p)
        return [self.r2cp(x * tmp, p) for x in acc]

    def advect_p(self, a, b, c, th, p):
        tmp = 1.0 / (float(self.nx) * self.ny * self.nz) ** 2
        acc = 0.0
        for d, v in zip((1, 2, 3), (a, b, c)):
            acc = acc + self.c2rp(v, p) * self.c2rp(rnd(self.derivk(th, d), p), p)
        return self.r2cp(acc * tmp, p)

    def sol_project_p(self, a, b, c, p):
        a, b, c = rnd(a, p), rnd(b, p), rnd(c, p)
        with np.errstate(invalid="ignore", divide="ignore"):
            d = -1j * (self.KX * a + self.KY * b + self.KZ * c) / self.kk2
        d[0, 0, 0] = 0
        d = rnd(d, p)
        a = rnd(a - 1j * self.KX * d, p)
        b = rnd(b - 1j * self.KY * d, p)
        c = rnd(c - 1j * self.KZ * d, p)
        C1 = self.c2r_zp(c / self.nz, 64)  # wall values: FP64 sums of the spectrum
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
        pr = rnd(self.c2r_zp(d, p) / self.nz + rnd(A, p), p)
        A, Bp = rnd(self.r2c_z(A), p), rnd(self.r2c_z(Bp), p)  # FP64 harmonic spectra, rounded
        return rnd(a - 1j * self.KX * A, p), rnd(b - 1j * self.KY * A, p), rnd(c - Bp, p), pr

    def imposebc_p(self, vx, vy, vz, pr, o, ord, p):
        vx, vy = self.c2r_zp(vx, p), self.c2r_zp(vy, p)
        vx[:, :, : self.nzp] /= self.nz
        vy[:, :, : self.nzp] /= self.nz
        tmp = 1.0 / o if o == ord else (o + 1) / o
        for ind in (0, self.nzp - 1):
            vx[:, :, ind] = 1j * self.kx[:, None] * pr[:, :, ind] * tmp
            vy[:, :, ind] = 1j * self.ky[None, :] * pr[:, :, ind] * tmp
            vx[0, 0, ind] = 0
            vy[0, 0, ind] = 0
        return self.r2c_zp(rnd(vx, p), p), self.r2c_zp(rnd(vy, p), p), vz

    def s_imposebc_p(self, th, p):
        t = self.c2r_zp(th, p)
        t[:, :, : self.nzp] /= self.nz
        t[:, :, 0] = 0
        t[:, :, self.nzp - 1] = 0
        return self.r2c_zp(rnd(t, p), p)

    def bouss_stage_p(self, P, o, v, th, pr, Cs, C7, F):
        rmp = 1.0 / o
        pn = F["nl"]
        N = self.gradre_p(*v, pn)
        N8 = self.advect_p(*v, th, pn)
        N[2] = rnd(N[2] - P["xmom"] * th, pn)
        N8 = rnd(N8 - P["xtemp"] * v[2], pn)
        N = [rnd(self.fc_filter(x), pn) for x in N]
        N8 = rnd(self.fc_filter(N8), pn)
        pu = F["upd"]
        vn = [rnd(Cc + P["dt"] * (P["nu"] * (-self.kk2 * x) - n) * rmp, pu) for x, n, Cc in zip(v, N, Cs)]
        th = rnd(C7 + P["dt"] * (P["kappa"] * (-self.kk2 * th) - N8) * rmp, pu)
        vx, vy, vz = self.imposebc_p(*vn, pr, o, P["ord"], F["R"])
        vx, vy, vz, pr = self.sol_project_p(vx, vy, vz, F["proj"])
        th = self.s_imposebc_p(th, F["R"])
        th = rnd(self.fc_filter(th), F["filt"])
        ph = F["hack"]
        th = self.r2cp(self.c2rp(th, ph) / self.nx / self.ny / self.nz, ph)
        ps = F["state"]
        return [rnd(x, ps) for x in (vx, vy, vz)], rnd(th, ps), rnd(pr, ps)


PARAMS = dict(dt=1e-5, nu=1e-4, kappa=1e-4, xmom=1.0, xtemp=1.0, ord=2)
FP64 = dict(nl=64, upd=64, R=64, proj=64, filt=64, hack=64, state=64)


def initial_theta(g, seed=20261203, amp=1e-3):
    rng = np.random.default_rng(seed)
    xi = rng.uniform(-1.0, 1.0, size=(g.nzp, g.ny, g.nx))
    z = g.z[: g.nzp]
    full = np.zeros((g.nz, g.ny, g.nx))
    full[: g.nzp] = amp * xi * (z * (g.Lz - z))[:, None, None]
    return g.r2c(full)


def run(g, flags, nsteps, checks, P=PARAMS):
    th = initial_theta(g)
    zero = np.zeros_like(th)
    v, pr = [zero.copy(), zero.copy(), zero.copy()], zero.copy()
    out = {}
    for s in range(1, nsteps + 1):
        Cs = [x.copy() for x in v]
        C7 = th.copy()
        for o in range(P["ord"], 0, -1):
            v, th, pr = g.bouss_stage_p(P, o, v, th, pr, Cs, C7, flags)
        if s in checks:
            out[s] = [g.c2r(x.copy())[: g.nzp] for x in v + [th]]
    return out


def variant(spec):
    if spec == "all32":
        return {k: 32 for k in FP64}
    f = dict(FP64)
    for kv in spec.split(","):
        k, val = kv.split("=")
        f[k] = int(val)
    return f


def relerr(a, b):
    return [float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)) for x, y in zip(a, b)]


def study(nxy, nsteps, specs):
    g = PG(nxy, nxy, 513 + 25, 25, 5, 1.0, 1.0, 1.0)
    checks = sorted({10, 100, 300, 1000, nsteps} & set(range(1, nsteps + 1)))
    ref = run(g, FP64, nsteps, checks)
    rows = []
    for spec in specs:
        res = run(g, variant(spec), nsteps, checks)
        for s in checks:
            rows.append({"variant": spec, "step": s, "rel_l2": relerr(res[s], ref[s])})
    return rows


if __name__ == "__main__":
    nxy = int(sys.argv[1]) if len(sys.argv) > 1 else 16
    nsteps = int(sys.argv[2]) if len(sys.argv) > 2 else 100
    specs = sys.argv[3].split(";") if len(sys.argv) > 3 else ["all32", "nl=32"]
    for row in study(nxy, nsteps, specs):
        print(json.dumps({"variant": row["variant"], "step": row["step"],
                          "rel_l2": ["%.2e" % e for e in row["rel_l2"]]}), flush=True)
