"""A precision form against the plain FP64 form, both on the GPU.

Forms: nl32 (default) keeps the state and everything that carries it through a z transform in
FP64 and runs the nonlinear term in FP32 (Solver(..., nl_fp32=True) on an FP64 plan); fp32 is
the FP32-bulk plan (every transform FP32, FP64 only for the continuation arithmetic, the wall
solve and the reductions).

The same seeded case runs through both forms; at each checkpoint the relative L2 error of every
state field is reported on the physical grid (rows z < nzp):

    err(f) = ||f_fp32 - f_fp64||_2 / ||f_fp64||_2

velocity and temperature in real space (c2r of both states in FP64), the pressure potential in
the mixed (z, ky, kx) domain where the solver keeps it.  The FP64 form itself matches the FP64
CPU restatement of the reference to 1e-10 (tests/test_gpu_configs.py), so this is the precision
form's error against the reference algorithm.

    python -m specter_gb300.precision_study --case channel256 --check 100,1000
    python -m specter_gb300.precision_study --case bouss512 --check 10,100,1000 [--form fp32]

Cases (seeded initial fields of specter_gb300.initial):
  channel64   HD channel 64^2 x 65 (+25), Lz = 2, RK2, dt 1e-4, nu 1e-3, |k| <= 8, amp 0.05
  channel256  HD channel 256^2 x 257 (+25), Lz = 2, RK4, dt 2e-5, nu 2e-4, |k| <= 32, amp 0.1
  bouss512    Rayleigh-Benard 512^2 x 513 (+25), Lz = 1, RK2, dt 1e-5, nu = kappa = 1e-4
Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

CASES = {
    "channel64": dict(nx=64, ny=64, nzp=65, Lz=2.0, solver="HD", ord=2, dt=1e-4, nu=1e-3, kappa=0.0,
                      amp=0.05, kmax=8),
    "channel256": dict(nx=256, ny=256, nzp=257, Lz=2.0, solver="HD", ord=4, dt=2e-5, nu=2e-4, kappa=0.0,
                       amp=0.1, kmax=32),
    "bouss512": dict(nx=512, ny=512, nzp=513, Lz=1.0, solver="BOUSS", ord=2, dt=1e-5, nu=1e-4, kappa=1e-4,
                     amp=1e-3, kmax=0),
}
SEED = 20261203


def make_solver(api, initial, c, precision, fused=True, nl_fp32=False):
    nz = c["nzp"] + 25
    plan = api.Plan((c["nx"], c["ny"], nz), (0, 0, 25), (0, 0, 5), (1.0, 1.0, c["Lz"]), precision=precision)
    bouss = c["solver"] == "BOUSS"
    s = api.Solver(plan, api.BOUSS if bouss else api.HD, ord=c["ord"], dt=c["dt"], nu=c["nu"],
                   kappa=c["kappa"], fused=fused, nl_fp32=nl_fp32)
    if bouss:
        th = initial.convection_theta(plan, seed=SEED, amp=c["amp"])
        s.th.copy_from(initial.to_spectral(plan, [th])[0])
        for f in (s.vx, s.vy, s.vz, s.pr):
            f.zero()
    else:
        v = initial.channel_velocity(plan, seed=SEED, amp=c["amp"], kmax=c["kmax"])
        for f, sp in zip((s.vx, s.vy, s.vz), initial.to_spectral(plan, v)):
            f.copy_from(sp)
        s.pr.zero()
    plan.synchronize()
    return plan, s


def physical(api, p64, scratch_c, scratch_r, data):
    """Real-space rows z < nzp of a spectral field given as a host array (FP64 c2r)."""
    scratch_c.upload(np.ascontiguousarray(data, dtype=np.complex128))
    api.fftp3d_complex_to_real(p64, scratch_c, scratch_r)
    return scratch_r.download()[: p64.nzp]


def compare(api, p64, s32, s64, names, scratch):
    out = {}
    f32 = [f for f in (s32.vx, s32.vy, s32.vz, s32.th) if f is not None]
    f64 = [f for f in (s64.vx, s64.vy, s64.vz, s64.th) if f is not None]
    for name, a, b in zip(names, f32, f64):
        ra = physical(api, p64, *scratch, a.download())
        rb = physical(api, p64, *scratch, b.download())
        nb = np.linalg.norm(rb)
        out[name] = float(np.linalg.norm(ra - rb) / nb) if nb > 0 else float(np.linalg.norm(ra))
    pa, pb = s32.pr.download()[..., : p64.nzp].astype(np.complex128), s64.pr.download()[..., : p64.nzp]
    nb = np.linalg.norm(pb)
    out["pr"] = float(np.linalg.norm(pa - pb) / nb) if nb > 0 else float(np.linalg.norm(pa))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="channel256", choices=sorted(CASES))
    ap.add_argument("--check", default="100,1000", help="comma-separated step counts")
    ap.add_argument("--fused", type=int, default=1)
    ap.add_argument("--form", default="nl32", choices=["nl32", "fp32"],
                    help="nl32: FP64 state, FP32 nonlinear term (nl_fp32); fp32: the FP32-bulk plan")
    args = ap.parse_args(argv)
    from specter_gb300 import api, initial
    c = CASES[args.case]
    checks = sorted({int(x) for x in args.check.split(",")})
    if args.form == "nl32":
        p32, s32 = make_solver(api, initial, c, api.FP64, True, nl_fp32=True)
    else:
        p32, s32 = make_solver(api, initial, c, api.FP32, bool(args.fused))
    p64, s64 = make_solver(api, initial, c, api.FP64, bool(args.fused))
    names = ["vx", "vy", "vz"] + (["th"] if c["solver"] == "BOUSS" else [])
    scratch = (p64.field(api.COMPLEX), p64.field(api.REAL))
    done, t32, t64, rows = 0, 0.0, 0.0, []
    for n in checks:
        k = n - done
        t0 = time.perf_counter()
        s32.step(k)
        p32.synchronize()
        t1 = time.perf_counter()
        s64.step(k)
        p64.synchronize()
        t2 = time.perf_counter()
        t32 += t1 - t0
        t64 += t2 - t1
        done = n
        s32.check()
        s64.check()
        errs = compare(api, p64, s32, s64, names, scratch)
        rows.append({"steps": n, "rel_l2": errs, "max": max(errs[k_] for k_ in names)})
        print(json.dumps({"progress": rows[-1]}), flush=True)
    pts = c["nx"] * c["ny"] * c["nzp"] * c["ord"] * done
    line = {"case": args.case, "form": args.form, "config": c, "seed": SEED, "fused": bool(args.fused), "checkpoints": rows,
            "form_mpts_stages_per_s": round(pts / t32 / 1e6, 2), "fp64_mpts_stages_per_s": round(pts / t64 / 1e6, 2),
            "metric": "relative L2 on physical rows; pr in the mixed domain"}
    print(json.dumps(line), flush=True)
    return line


if __name__ == "__main__":
    main()
