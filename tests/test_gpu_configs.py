"""The plain FP64 channel configuration against the oracle: 64 x 64 x 65 (+25), no-slip walls,
nu = 1e-3, RK2, dt = 1e-4, 100 steps, seeded Poiseuille + solenoidal perturbation (|k| <= 8,
amplitude 0.05).  Velocity within 1e-10 relative L2; diagnostics (balance and no-slip files'
quantities) within 1e-10 relative."""
import numpy as np
import pytest

from conftest import make_pair, rel

pytestmark = pytest.mark.gpu

STEPS = 100


@pytest.fixture(scope="module")
def channel_run():
    from specter_gb300 import api, initial
    plan, g = make_pair(64, 64, 65, 2.0)
    real = initial.channel_velocity(plan, seed=20261203, amp=0.05, kmax=8)
    v0 = [g.fftp3d_real_to_complex(r) for r in real]
    pr0 = np.zeros(g.sshape, complex)
    kw = dict(dt=1e-4, nu=1e-3, ord=2)

    class Runs(dict):
        def __missing__(self, fused):
            s = api.Solver(plan, api.HD, fused=fused, **kw)
            for f, a in zip((s.vx, s.vy, s.vz, s.pr), v0 + [pr0]):
                f.upload(a)
            s.step(STEPS)
            self[fused] = (s, [f.download() for f in (s.vx, s.vy, s.vz, s.pr)])
            return self[fused]

    ref = g.run(g.params(**kw), STEPS, *v0, pr0)
    return plan, g, Runs(), ref


@pytest.mark.parametrize("fused", [False, True], ids=["refseq", "fused"])
def test_channel_state(channel_run, fused):
    plan, g, out, ref = channel_run
    s, got = out[fused]
    for a, b in zip(got[:3], ref[:3]):
        assert rel(a, b) < 1e-10
    nzp = g.nz - g.cz
    assert rel(got[3][:, :, :nzp], ref[3][:, :, :nzp]) < 1e-8


@pytest.mark.parametrize("fused", [False, True], ids=["refseq", "fused"])
def test_channel_diagnostics(channel_run, fused):
    """hdcheck (balance.txt) and vdiagnostic (noslip_diagnostic.txt) quantities."""
    from specter_gb300 import api
    plan, g, out, ref = channel_run
    s, _ = out[fused]
    v = ref[:3]
    f = (s.vx, s.vy, s.vz)
    assert api.energy(plan, *f, 1) == pytest.approx(g.energy(*v, 1), rel=1e-10)
    assert api.energy(plan, *f, 0) == pytest.approx(g.energy(*v, 0), rel=1e-10)
    assert api.helicity(plan, *f) == pytest.approx(g.helicity(*v), rel=1e-8, abs=1e-12)
    div = api.divergence(plan, *f)
    assert div == pytest.approx(g.divergence(*v), rel=1e-6, abs=1e-14)
    bt = api.bouncheck_z(plan, f[0], f[1])
    rt = g.bouncheck_z(v[0], v[1])
    assert bt == pytest.approx(rt, rel=1e-8, abs=1e-20)
    bn = api.bouncheck_z(plan, f[2])
    assert bn == pytest.approx(g.bouncheck_z(v[2]), rel=1e-6, abs=1e-20)
