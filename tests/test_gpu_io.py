"""Diagnostic files and raw snapshots against the FP64 oracle, through the C ABI.

The diagnostic values written to balance.txt / noslip_diagnostic.txt / scalar.txt /
scalar_constant_diagnostic.txt must equal the oracle's reductions of the same state to 1e-10;
snapshots must hold the oracle's physical fields to 1e-12 and restart must reproduce the state
to 1e-10."""
import os

import numpy as np
import pytest

from conftest import make_pair, rel

pytestmark = pytest.mark.gpu


def _channel(api, initial, plan, steps, bouss=False):
    if bouss:
        s = api.Solver(plan, api.BOUSS, ord=2, dt=1e-4, nu=1e-3, kappa=1e-3)
        th = initial.convection_theta(plan, seed=4, amp=1e-2)
        s.th.copy_from(initial.to_spectral(plan, [th])[0])
        v = initial.channel_velocity(plan, seed=5, amp=0.05, kmax=4)
        for f, sp in zip((s.vx, s.vy, s.vz), initial.to_spectral(plan, v)):
            f.copy_from(sp)
    else:
        s = api.Solver(plan, api.HD, ord=2, dt=1e-4, nu=1e-3)
        v = initial.channel_velocity(plan, seed=5, amp=0.05, kmax=4)
        for f, sp in zip((s.vx, s.vy, s.vz), initial.to_spectral(plan, v)):
            f.copy_from(sp)
    s.pr.zero()
    s.step(steps)
    return s


def _cols(path):
    return [[float(x.replace("D", "E")) for x in l.split()] for l in open(path)]


def test_diagnostic_files(tmp_path):
    from specter_gb300 import api, initial
    from specter_gb300.diagnostics import Diagnostics
    plan, g = make_pair(32, 24, 33, 2.0)
    s = _channel(api, initial, plan, 3, bouss=True)
    d = Diagnostics(plan, str(tmp_path))
    d.hdcheck(s.vx, s.vy, s.vz, t=4, dt=1e-4, hel=1)
    d.vdiagnostic(s.vx, s.vy, s.vz, t=4, dt=1e-4)
    d.pscheck(s.th, t=4, dt=1e-4)
    d.sdiagnostic(s.th, t=4, dt=1e-4)
    vx, vy, vz, th = (f.download() for f in (s.vx, s.vy, s.vz, s.th))
    z = np.zeros_like(vx)
    bal = _cols(tmp_path / "balance.txt")[0]
    assert bal[0] == pytest.approx(3e-4)
    assert bal[1] == pytest.approx(g.energy(vx, vy, vz, 1), rel=1e-10)
    assert bal[2] == pytest.approx(g.energy(vx, vy, vz, 0), rel=1e-10)
    assert bal[3] == pytest.approx(g.cross(vx, vy, vz, z, z, z, 1), abs=1e-300)
    hel = _cols(tmp_path / "helicity.txt")[0]
    assert hel[1] == pytest.approx(g.helicity(vx, vy, vz), rel=1e-9, abs=1e-20)
    ns = _cols(tmp_path / "noslip_diagnostic.txt")[0]
    t1, t2 = g.bouncheck_z(vx, vy)
    t3, t4 = g.bouncheck_z(vz)
    ref = [3e-4, g.divergence(vx, vy, vz), t1, t2, t3, t4]
    for got, want in zip(ns, ref):
        assert got == pytest.approx(want, rel=5e-7, abs=1e-30)  # E13.6 keeps 7 digits
    sc = _cols(tmp_path / "scalar.txt")[0]
    assert sc[1] == pytest.approx(g.variance(th, 1), rel=1e-10)
    assert sc[2] == pytest.approx(g.variance(th, 0), rel=1e-10)
    sb = _cols(tmp_path / "scalar_constant_diagnostic.txt")[0]
    b1, b2 = g.bouncheck_z(th)
    assert sb[1] == pytest.approx(b1, rel=5e-7, abs=1e-30) and sb[2] == pytest.approx(b2, rel=5e-7, abs=1e-30)
    line = open(tmp_path / "balance.txt").read().rstrip("\n")
    assert len(line) == 13 + 23 + 23 + 24


def test_snapshot_and_restart(tmp_path):
    from specter_gb300 import api, checkpoint, initial
    plan, g = make_pair(32, 24, 33, 2.0)
    dt = 1e-4
    s = _channel(api, initial, plan, 2, bouss=True)
    paths = checkpoint.write(s, str(tmp_path), 7, dt, outs=1)
    assert os.path.basename(paths[0]) == "wx.0007.out"
    N = plan.nx * plan.ny * plan.nz
    vx = s.vx.download()
    ref = g.fftp3d_complex_to_real(vx / N)[: plan.nzp]
    got = np.fromfile(tmp_path / "vx.0007.out", dtype=np.float64).reshape(plan.nzp, plan.ny, plan.nx)
    assert rel(got, ref) < 1e-12
    pref = g.fftp2d_complex_to_real_xy(s.pr.download() / (plan.nx * plan.ny * dt))[: plan.nzp]
    pgot = np.fromfile(tmp_path / "pr.0007.out", dtype=np.float64).reshape(plan.nzp, plan.ny, plan.nx)
    assert rel(pgot, pref) < 1e-12
    # restart: the reference re-transforms the physical planes (the continuation rows are rebuilt
    # from the wall-adjacent points), so the restarted state is the r2c of the files
    s2 = api.Solver(plan, api.BOUSS, ord=2, dt=dt, nu=1e-3, kappa=1e-3)
    checkpoint.read(s2, str(tmp_path), 7, dt)

    def padded(name):
        r = np.zeros(g.rshape)
        r[: plan.nzp] = np.fromfile(tmp_path / f"{name}.0007.out", dtype=np.float64).reshape(plan.nzp, plan.ny, plan.nx)
        return r

    for name, f in zip(("vx", "vy", "vz", "th"), (s2.vx, s2.vy, s2.vz, s2.th)):
        assert rel(f.download(), g.fftp3d_real_to_complex(padded(name))) < 1e-11, name
    pr_ref = g.fftp2d_real_to_complex_xy(padded("pr"))[..., : plan.nzp] * dt
    assert rel(s2.pr.download()[..., : plan.nzp], pr_ref) < 1e-11
    # and the physical fields survive the round trip
    back = g.fftp3d_complex_to_real(s2.vx.download() / N)[: plan.nzp]
    assert rel(back, ref) < 1e-10
