"""Snapshots and restart in the reference's raw output format.

File odir/<name>.<NNNN>.out holds one field on the physical grid only (nz - Cz planes), as raw
native-endian reals of the run's precision in Fortran order R(nx, ny, nz - Cz)
(src/mpiio/binary_io.f90:165-226 with the I/O plan of src/specter.fpp:291).  Written fields
(src/specter.fpp:1005-1068):
  vx, vy, vz, th   c2r of the spectral field times 1/(nx ny nz)
  wx, wy, wz       (outs >= 1) c2r of curl(v) times 1/(nx ny nz)
  pr               the pressure p = p'/dt: 2-D (x, y) c2r of the mixed-domain p' times 1/(nx ny dt)
Restart (src/specter.fpp:885-935) reads them back: r2c for vx, vy, vz, th; for pr a 2-D r2c and
p' = p * dt on the physical planes.  Transforms run on the GPU; only the (x, y)-normalisation
multiply happens on the host.
"""
from __future__ import annotations

import os

import numpy as np


def _path(d, name, index):
    return os.path.join(d, f"{name}.{index:04d}.out" if isinstance(index, int) else f"{name}.{index}.out")


def _scaled_real(api, plan, spectral, scale, two_d=False):
    """real physical planes of (spectral * scale) through the GPU c2r (input left untouched)."""
    tmp = plan.field(api.COMPLEX, data=(spectral.download() * scale).astype(plan.cdtype))
    out = plan.field(api.REAL)
    if two_d:
        api.fftp2d_complex_to_real_xy(plan, tmp, out)
    else:
        api.fftp3d_complex_to_real(plan, tmp, out)
    r = out.download()[: plan.nzp]
    tmp.close()
    out.close()
    return np.ascontiguousarray(r)


def write(solver, odir, index, dt, outs=0):
    """Writes the solver state as the reference's output set number `index`; returns the paths."""
    from specter_gb300 import api
    plan = solver.plan
    os.makedirs(odir, exist_ok=True)
    rmp = 1.0 / (plan.nx * plan.ny * plan.nz)
    paths = []
    names = [("vx", solver.vx), ("vy", solver.vy), ("vz", solver.vz)]
    if outs >= 1:
        c = [plan.field() for _ in range(3)]
        api.curlk(plan, solver.vy, solver.vz, c[0], 1)
        api.curlk(plan, solver.vx, solver.vz, c[1], 2)
        api.curlk(plan, solver.vx, solver.vy, c[2], 3)
        names = list(zip(("wx", "wy", "wz"), c)) + names
    for name, f in names:
        p = _path(odir, name, index)
        _scaled_real(api, plan, f, rmp).tofile(p)
        paths.append(p)
    p = _path(odir, "pr", index)
    _scaled_real(api, plan, solver.pr, 1.0 / (plan.nx * plan.ny * dt), two_d=True).tofile(p)
    paths.append(p)
    if solver.th is not None:
        p = _path(odir, "th", index)
        _scaled_real(api, plan, solver.th, rmp).tofile(p)
        paths.append(p)
    return paths


def _read_real(plan, path):
    a = np.fromfile(path, dtype=plan.rdtype)
    if a.size != plan.nx * plan.ny * plan.nzp:
        raise ValueError(f"{path}: {a.size} values, expected nx*ny*(nz-Cz) = {plan.nx * plan.ny * plan.nzp}")
    r = np.zeros(plan.rshape, dtype=plan.rdtype)
    r[: plan.nzp] = a.reshape(plan.nzp, plan.ny, plan.nx)
    return r


def read(solver, idir, index, dt):
    """Loads output set `index` into the solver state (the reference's restart with stat > 0)."""
    from specter_gb300 import api
    plan = solver.plan
    targets = [("vx", solver.vx), ("vy", solver.vy), ("vz", solver.vz)]
    if solver.th is not None:
        targets.append(("th", solver.th))
    for name, f in targets:
        api.fftp3d_real_to_complex(plan, plan.field(api.REAL, data=_read_real(plan, _path(idir, name, index))), f)
    tmp = plan.field(api.COMPLEX)
    api.fftp2d_real_to_complex_xy(plan, plan.field(api.REAL, data=_read_real(plan, _path(idir, "pr", index))), tmp)
    pr = tmp.download()
    pr[..., : plan.nzp] *= dt
    pr[..., plan.nzp:] = 0
    solver.pr.upload(pr)
    plan.synchronize()
