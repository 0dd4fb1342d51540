"""GPU parity: every reference routine of the hot path, through the C ABI, against the FP64 oracle.

FP64 tolerances (relative L2): transforms 1e-12 and stages 1e-11 — the FC-Gram continuation
amplifies summation-order rounding by up to ~1e4 (|dir| <= 3.5e3), so two correct FP64
implementations differ at ~1e-13..1e-12.  The pressure potential pr (= dt*p) after a stage is
-i k.v/k^2 of a velocity that was projected one stage earlier: k.v is a small residual, so
pr's relative error is the velocity's error divided by that residual; it is held to 1e-8.
"""
import numpy as np
import pytest

from conftest import make_pair, rel, smooth_spectral

pytestmark = pytest.mark.gpu

GRIDS = [
    (16, 16, 33, 2.0),   # NZ = 58 = 2*29 (Bluestein)
    (48, 12, 29, 1.0),   # nx/2 = 24, ny = 12 (radix 3), NZ = 54
    (32, 20, 129, 1.0),  # ny = 20 (radix 5), NZ = 154 = 2*7*11
    (64, 64, 65, 2.0),   # the plain-FP64 channel grid, NZ = 90
    (32, 32, 513, 1.0),  # the Rayleigh-Benard z grid, NZ = 538 = 2*269 (Bluestein 1080)
]


@pytest.fixture(scope="module", params=GRIDS, ids=lambda g: "x".join(map(str, g[:3])))
def pair(request):
    nx, ny, nzp, Lz = request.param
    return make_pair(nx, ny, nzp, Lz)


def rand_c(g, rng, scale=1.0):
    return (rng.standard_normal(g.sshape) + 1j * rng.standard_normal(g.sshape)) * scale


def test_field_round_trip(pair):
    plan, g = pair
    rng = np.random.default_rng(1)
    a = rand_c(g, rng)
    f = plan.field(data=a)
    assert np.array_equal(f.download(), a)
    r = rng.standard_normal(g.rshape)
    fr = plan.field(1, data=r)
    assert np.array_equal(fr.download(), r)


def test_fftp_transforms(pair):
    from specter_gb300 import api
    plan, g = pair
    rng = np.random.default_rng(2)
    r = rng.standard_normal(g.rshape)
    out = plan.field()
    api.fftp3d_real_to_complex(plan, plan.field(1, data=r), out)
    assert rel(out.download(), g.fftp3d_real_to_complex(r)) < 1e-12

    c = rand_c(g, rng)
    cin, rout = plan.field(data=c), plan.field(1)
    api.fftp3d_complex_to_real(plan, cin, rout)
    assert rel(rout.download(), g.fftp3d_complex_to_real(c)) < 1e-12

    out2 = plan.field()
    api.fftp2d_real_to_complex_xy(plan, plan.field(1, data=r), out2)
    assert rel(out2.download(), g.fftp2d_real_to_complex_xy(r)) < 1e-13
    rout2 = plan.field(1)
    cin2 = plan.field(data=c)
    api.fftp2d_complex_to_real_xy(plan, cin2, rout2)
    assert rel(rout2.download(), g.fftp2d_complex_to_real_xy(c)) < 1e-13
    assert np.array_equal(cin2.download(), c)  # fftp2d_complex_to_real_xy leaves its input intact

    z1 = plan.field(data=c)
    api.fftp1d_real_to_complex_z(plan, z1)
    assert rel(z1.download(), g.fftp1d_real_to_complex_z(c)) < 1e-12
    z2 = plan.field(data=c)
    api.fftp1d_complex_to_real_z(plan, z2)
    assert rel(z2.download(), g.fftp1d_complex_to_real_z(c)) < 1e-13


def test_spectral_operators(pair):
    from specter_gb300 import api
    plan, g = pair
    rng = np.random.default_rng(3)
    a, b = rand_c(g, rng), rand_c(g, rng)
    fa, fb, fo = plan.field(data=a), plan.field(data=b), plan.field()
    for d in (1, 2, 3):
        api.derivk(plan, fa, fo, d)
        assert rel(fo.download(), g.derivk(a, d)) < 1e-15
        api.curlk(plan, fa, fb, fo, d)
        assert rel(fo.download(), g.curlk(a, b, d)) < 1e-15
    api.laplak(plan, fa, fo)
    assert rel(fo.download(), g.laplak(a)) < 1e-15
    ff = plan.field(data=a)
    api.fc_filter(plan, ff)
    assert rel(ff.download(), g.fc_filter(a)) < 1e-15


def test_nonlinear_terms(pair):
    from specter_gb300 import api
    plan, g = pair
    rng = np.random.default_rng(4)
    v = [smooth_spectral(g, rng) for _ in range(3)]
    th = smooth_spectral(g, rng)
    fv = [plan.field(data=x) for x in v]
    out = [plan.field() for _ in range(3)]
    api.gradre(plan, *fv, *out)
    for got, ref in zip(out, g.gradre(*v)):
        assert rel(got.download(), ref) < 1e-11
    fe = plan.field()
    api.advect(plan, *fv, plan.field(data=th), fe)
    assert rel(fe.download(), g.advect(*v, th)) < 1e-11


def test_diagnostics(pair):
    from specter_gb300 import api
    plan, g = pair
    rng = np.random.default_rng(5)
    v = [smooth_spectral(g, rng) for _ in range(6)]
    f = [plan.field(data=x) for x in v]
    for kin in (0, 1, 2):
        assert api.energy(plan, *f[:3], kin) == pytest.approx(g.energy(*v[:3], kin), rel=1e-11)
    assert api.helicity(plan, *f[:3]) == pytest.approx(g.helicity(*v[:3]), rel=1e-10, abs=1e-14)
    for kin in (0, 1):
        assert api.cross(plan, *f, kin) == pytest.approx(g.cross(*v, kin), rel=1e-10, abs=1e-14)
    assert api.divergence(plan, *f[:3]) == pytest.approx(g.divergence(*v[:3]), rel=1e-11)
    for kin in (0, 1):
        assert api.variance(plan, f[0], kin) == pytest.approx(g.variance(v[0], kin), rel=1e-11)
    assert api.product(plan, f[0], f[1]) == pytest.approx(g.product(v[0], v[1]), rel=1e-10, abs=1e-14)
    bt = api.bouncheck_z(plan, f[0], f[1])
    assert bt == pytest.approx(g.bouncheck_z(v[0], v[1]), rel=1e-11)
    assert api.bouncheck_z(plan, f[2]) == pytest.approx(g.bouncheck_z(v[2]), rel=1e-11)


@pytest.mark.parametrize("bctarget", [1, 0])
def test_sol_project(pair, bctarget):
    from specter_gb300 import api
    plan, g = pair
    rng = np.random.default_rng(6)
    v = [smooth_spectral(g, rng) for _ in range(3)]
    f = [plan.field(data=x) for x in v]
    d = plan.field()
    api.sol_project(plan, *f, d, bctarget, 0, 0)
    ra, rb, rc, rd = g.sol_project(*v, bctarget, 0, 0)
    for got, ref in zip(f, (ra, rb, rc)):
        assert rel(got.download(), ref) < 1e-11
    nzp = g.nz - g.cz
    assert rel(d.download()[:, :, :nzp], rd[:, :, :nzp]) < 1e-11


def test_unsupported_bc_is_an_error(pair):
    from specter_gb300 import api, SpecterError
    plan, g = pair
    f = [plan.field() for _ in range(4)]
    with pytest.raises(SpecterError) as e:
        api.sol_project(plan, *f, 1, 2, 2)
    assert e.value.code == 3


@pytest.mark.parametrize("rki", [2, 1])
def test_imposebc(pair, rki):
    from specter_gb300 import api
    plan, g = pair
    rng = np.random.default_rng(7)
    v = [smooth_spectral(g, rng) for _ in range(4)]
    pr = g.fftp1d_complex_to_real_z(smooth_spectral(g, rng, amp=1e-2)) / g.nz
    f = [plan.field(data=x) for x in v[:3]]
    fp = plan.field(data=pr)
    api.v_imposebc_and_project(plan, *f, fp, rki, 2, (0.1, -0.2), (0.3, 0.05))
    ref = g.v_imposebc_and_project(*v[:3], pr, rki, 2, (0.1, -0.2), (0.3, 0.05))
    for got, r in zip(f, ref[:3]):
        assert rel(got.download(), r) < 1e-11
    nzp = g.nz - g.cz
    assert rel(fp.download()[:, :, :nzp], ref[3][:, :, :nzp]) < 1e-11
    ft = plan.field(data=v[3])
    api.s_imposebc(plan, ft)
    assert rel(ft.download(), g.s_imposebc(v[3])) < 1e-11


OMEGA = (0.3, -0.7, 2.0)


@pytest.mark.parametrize("solver", [0, 1, 2], ids=["HD", "BOUSS", "ROTBOUSS"])
@pytest.mark.parametrize("fused", [False, True, "one-kernel"], ids=["refseq", "fused", "fused1"])
def test_rk_step(pair, solver, fused):
    from specter_gb300 import api
    plan, g = pair
    api.set_option(plan, "velocity_split", 0 if fused == "one-kernel" else 1)
    fused = bool(fused)
    rng = np.random.default_rng(8 + solver)
    v = [smooth_spectral(g, rng, amp=0.3) for _ in range(3)]
    th = smooth_spectral(g, rng, amp=0.3)
    pr = g.fftp1d_complex_to_real_z(smooth_spectral(g, rng, amp=1e-3)) / g.nz
    kw = dict(dt=1e-3, nu=1e-2, ord=2, kappa=5e-3)
    s = api.Solver(plan, solver, fused=fused, omega=OMEGA if solver == 2 else (0.0, 0.0, 0.0), **kw)
    for fld, a in zip((s.vx, s.vy, s.vz), v):
        fld.upload(a)
    s.pr.upload(pr)
    if solver >= 1:
        s.th.upload(th)
    s.step(2)
    p = g.params(**kw)
    ref = g.run(p, 2, *v, pr, th=th if solver >= 1 else None, omega=OMEGA if solver == 2 else None)
    got = [f.download() for f in (s.vx, s.vy, s.vz)] + ([s.th.download()] if solver >= 1 else [])
    for a, b in zip(got, ref[: len(got)]):
        assert rel(a, b) < 1e-11
    nzp = g.nz - g.cz
    assert rel(s.pr.download()[:, :, :nzp], ref[-1][:, :, :nzp]) < 1e-8


def test_fields_batched_transfer():
    """specter_fields_upload / specter_fields_download move several fields like the single-field
    calls (pipelined through two staging buffers)."""
    from specter_gb300 import api
    plan = api.Plan((24, 16, 40), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 1.0), precision=1)
    rng = np.random.default_rng(3)
    data = [(rng.standard_normal(plan.sshape) + 1j * rng.standard_normal(plan.sshape)).astype(np.complex64)
            for _ in range(5)]
    fields = [plan.field() for _ in range(5)]
    api.fields_upload(fields, [d.ctypes.data for d in data])
    plan.synchronize()
    for f, d in zip(fields, data):
        assert np.array_equal(f.download(), d)
    out = [np.empty_like(d) for d in data]
    for f in fields:
        f.zero()
    for f, d in zip(fields, data):
        f.upload(d)
    api.fields_download(fields, [o.ctypes.data for o in out])
    for o, d in zip(out, data):
        assert np.array_equal(o, d)


def test_plan_limits():
    """Shapes the kernels cannot index (fields of 2^32 elements or more) or continue (d > 9) are
    refused at plan creation, before any allocation."""
    from specter_gb300 import SpecterError, api
    with pytest.raises(SpecterError) as e:
        api.Plan((8192, 8192, 4096 + 25), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 1.0), precision=1)
    assert e.value.code == 1
    with pytest.raises(SpecterError) as e:
        api.Plan((16, 16, 64), (0, 0, 25), (0, 0, 10), (1.0, 1.0, 1.0), precision=1)
    assert e.value.code == 1


def test_bouss_step_128x128x513():
    """One FP64 RK2 step of the Rayleigh-Benard case on a 128 x 128 x 513 (+25) grid against the
    oracle: fused stage kernels and the reference call sequence (bouss_rkstep2.f90:1-59)."""
    from specter_gb300 import api, initial
    plan, g = make_pair(128, 128, 513, 1.0)
    th = g.fftp3d_real_to_complex(initial.convection_theta(plan, seed=20261203, amp=1e-3))
    rng = np.random.default_rng(9)
    v = [smooth_spectral(g, rng, amp=1e-3) for _ in range(3)]
    pr = np.zeros(g.sshape, complex)
    kw = dict(dt=1e-5, nu=1e-4, kappa=1e-4, ord=2)
    ref = g.run(g.params(**kw), 1, *v, pr, th=th)
    for fused in (True, False):
        s = api.Solver(plan, api.BOUSS, fused=fused, **kw)
        for f, a in zip((s.vx, s.vy, s.vz, s.th, s.pr), v + [th, pr]):
            f.upload(a)
        s.step(1)
        got = [f.download() for f in (s.vx, s.vy, s.vz, s.th)]
        for a, b in zip(got, ref[:4]):
            assert rel(a, b) < 1e-11, fused
        s.close()
