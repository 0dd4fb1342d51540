"""The precision form (nl_fp32: FP64 state, FP32 nonlinear term) and the plain FP64 form at the
headline z length (nz = 513 physical + 25 continuation = 538 = 2*269, Bluestein), through the C
ABI, against the FP64 oracle.

Why this split of precisions: the FC-Gram continuation multiplies rounding in the 2d
wall-adjacent rows by up to sum|dir| = 9.5e3, and every operation that carries the state through
a z transform (the wall round trips of v_imposebc_and_project and s_imposebc, the projection,
fc_filter of theta and its c2r/r2c round trip) feeds those rows.  In FP32 each of them alone
costs 1e-5..4e-4 relative error after 100 Rayleigh-Benard steps.  The nonlinear term enters the
state multiplied by dt, so its FP32 rounding stays below the gate: the form keeps the nonlinear
term (its transforms and products) in FP32 and everything else in FP64.

Rayleigh-Benard grid 32 x 32 x 513 (+25): cfg3's z grid and physics (Lz = 1, nu = kappa = 1e-4,
dt = 1e-5, RK2, theta' = 1e-3 U(-1,1) z(1-z), v = 0) on a small periodic plane.
"""
import numpy as np
import pytest

from conftest import make_pair, rel

pytestmark = pytest.mark.gpu

STEPS = 20
SEED = 20261203


@pytest.fixture(scope="module")
def convection():
    from specter_gb300 import api, initial
    plan, g = make_pair(32, 32, 513, 1.0)
    th = initial.convection_theta(plan, seed=SEED, amp=1e-3)
    th0 = g.fftp3d_real_to_complex(th)
    zero = np.zeros(g.sshape, complex)
    kw = dict(dt=1e-5, nu=1e-4, kappa=1e-4, ord=2)
    p = g.params(**kw)
    ref = g.run(p, STEPS, zero, zero, zero, zero, th=th0)

    def run(**opts):
        s = api.Solver(plan, api.BOUSS, **kw, **opts)
        for f, a in zip((s.vx, s.vy, s.vz, s.th, s.pr), (zero, zero, zero, th0, zero)):
            f.upload(a)
        s.step(STEPS)
        out = [f.download() for f in (s.vx, s.vy, s.vz, s.th, s.pr)]
        s.close()
        return out

    return plan, g, ref, run


def _errors(g, got, ref):
    """relative L2 on the physical grid (c2r of both spectra, rows z < nzp)"""
    nzp = g.nz - g.cz
    out = []
    for a, b in zip(got[:4], [ref[0], ref[1], ref[2], ref[3]]):
        ra, rb = g.fftp3d_complex_to_real(a)[:nzp], g.fftp3d_complex_to_real(b)[:nzp]
        out.append(rel(ra, rb))
    return out


def test_fp64_bouss_nz538(convection):
    """Plain FP64, fused and reference call sequence, at NZ = 538."""
    plan, g, ref, run = convection
    for fused in (True, False):
        got = run(fused=fused)
        for a, b in zip(got[:4], ref[:4]):
            assert rel(a, b) < 1e-11, fused
        assert rel(got[4][..., : g.nz - g.cz], ref[4][..., : g.nz - g.cz]) < 1e-8, fused


def test_nl_fp32_bouss_nz538(convection):
    """The precision form after 20 steps: theta (which the FP32 nonlinear term reaches only
    through v.grad theta with v ~ 1e-8) to 1e-9, the velocity (driven by buoyancy from rest, so
    its error is relative to a small field) to 5e-6."""
    plan, g, ref, run = convection
    got = run(fused=True, nl_fp32=True)
    e = _errors(g, got, ref)
    nzp = g.nz - g.cz
    epr = rel(got[4][..., :nzp], ref[4][..., :nzp])
    print("nl_fp32 vs oracle after %d steps: vx %.2e vy %.2e vz %.2e th %.2e pr %.2e" % (STEPS, *e, epr))
    assert max(e[:3]) < 5e-6
    assert e[3] < 1e-9


@pytest.mark.parametrize("split,pair", [(1, 0), (0, 0), (1, 1)], ids=["split", "one_kernel", "split_pairs"])
def test_nl_fp32_engines_agree(convection, split, pair):
    """The float-float column kernels on the three-step Bluestein engine (the default at this z
    length) and on the generic Stockham engine: the same arithmetic up to float-float rounding
    (~1e-14 per transform), in the split velocity form and in the one-kernel form (whose tile
    widths and thread counts differ), with the three-step engine's kernels as one 576-thread
    block per SM or as two 288-thread blocks (pair).  Compared as spectra, where the FC-Gram continuation
    rows carry the wall-adjacent rounding amplified ~1e4x: after 20 steps both held to 1e-9
    (the physical-grid errors against the oracle stay at 1e-11)."""
    from specter_gb300 import api
    plan, g, ref, run = convection
    outs = []
    for engine in (1, 0):
        api.set_option(plan, "ff_engine", engine)
        api.set_option(plan, "velocity_split", split)
        api.set_option(plan, "ff_pair_proj", pair)
        api.set_option(plan, "ff_pair_cols", pair)
        outs.append(run(fused=True, nl_fp32=True))
    for name, v in (("ff_engine", 1), ("velocity_split", 1), ("ff_pair_proj", 0), ("ff_pair_cols", 0)):
        api.set_option(plan, name, v)
    d = [rel(a, b) for a, b in zip(outs[0][:4], outs[1][:4])]
    print("engines after %d steps (split %d): vx %.2e vy %.2e vz %.2e th %.2e" % (STEPS, split, *d))
    assert max(d) < 1e-9
    e = _errors(g, outs[0], ref)
    assert max(e[:3]) < 5e-6 and e[3] < 1e-9


@pytest.mark.parametrize("split", [1, 0], ids=["split", "one_kernel"])
def test_nl_fp32_window_corrections(convection, split):
    """The wall round trips of the float-float kernels as window corrections of the spectrum (the
    default) and as an inverse plus a forward transform: the same update in exact arithmetic
    (the round trip changes the column only on the 35 rows around the walls), so 20 steps agree to
    float-float rounding as amplified through the continuation (held to 1e-9 as spectra), and both
    stay at the oracle's 1e-11."""
    from specter_gb300 import api
    plan, g, ref, run = convection
    outs = []
    api.set_option(plan, "velocity_split", split)
    for zoom in (1, 0):
        api.set_option(plan, "ff_zoom", zoom)
        outs.append(run(fused=True, nl_fp32=True))
    api.set_option(plan, "ff_zoom", 1)
    api.set_option(plan, "velocity_split", 1)
    d = [rel(a, b) for a, b in zip(outs[0][:4], outs[1][:4])]
    e = _errors(g, outs[0], ref)
    print("window vs plain round trips after %d steps (split %d): vx %.2e vy %.2e vz %.2e th %.2e;"
          " vs oracle %s" % (STEPS, split, *d, " ".join("%.2e" % v for v in e)))
    assert max(d) < 1e-9
    assert max(e[:3]) < 5e-6 and e[3] < 1e-9


def test_nl_fp32_channel_nz282():
    """The channel z length of the 256^2 x 257 precision case (nz + C = 282 = 2 * 3 * 47, on the
    three-step engine as well): 16 x 16 x 257, Lz = 2, RK4, 20 steps against the oracle."""
    from specter_gb300 import api, initial
    plan, g = make_pair(16, 16, 257, 2.0)
    real = initial.channel_velocity(plan, seed=SEED, amp=0.1, kmax=4)
    v0 = [g.fftp3d_real_to_complex(r) for r in real]
    pr0 = np.zeros(g.sshape, complex)
    kw = dict(dt=2e-5, nu=2e-4, ord=4)
    ref = g.run(g.params(**kw), 20, *v0, pr0)
    s = api.Solver(plan, api.HD, fused=True, nl_fp32=True, **kw)
    for f, a in zip((s.vx, s.vy, s.vz, s.pr), v0 + [pr0]):
        f.upload(a)
    s.step(20)
    got = [f.download() for f in (s.vx, s.vy, s.vz)]
    s.close()
    e = [rel(a, b) for a, b in zip(got, ref[:3])]
    print("nl_fp32 channel nz 282 vs oracle after 20 steps: %.2e %.2e %.2e" % tuple(e))
    assert max(e) < 1e-7


def test_nl_fp32_channel():
    """The plain channel configuration (64 x 64 x 65, 100 RK2 steps) in the precision form."""
    from specter_gb300 import api, initial
    plan, g = make_pair(64, 64, 65, 2.0)
    real = initial.channel_velocity(plan, seed=SEED, amp=0.05, kmax=8)
    v0 = [g.fftp3d_real_to_complex(r) for r in real]
    pr0 = np.zeros(g.sshape, complex)
    kw = dict(dt=1e-4, nu=1e-3, ord=2)
    ref = g.run(g.params(**kw), 100, *v0, pr0)
    s = api.Solver(plan, api.HD, fused=True, nl_fp32=True, **kw)
    for f, a in zip((s.vx, s.vy, s.vz, s.pr), v0 + [pr0]):
        f.upload(a)
    s.step(100)
    got = [f.download() for f in (s.vx, s.vy, s.vz)]
    e = [rel(a, b) for a, b in zip(got, ref[:3])]
    print("nl_fp32 channel vs oracle after 100 steps: %.2e %.2e %.2e" % tuple(e))
    assert max(e) < 1e-5


@pytest.mark.parametrize("split", [1, 0], ids=["split", "one_kernel"])
@pytest.mark.parametrize("solver", [0, 1, 2], ids=["HD", "BOUSS", "ROTBOUSS"])
def test_nl_fp32_solvers_nz538(solver, split):
    """Every solver kind of the precision form at the headline z length (the three-step engine,
    the window corrections, the direct updates, and for ROTBOUSS the Coriolis term and the early
    end of the scalar kernel): two RK2 steps of smooth fields of order 0.3 against the FP64
    oracle.  The nonlinear term runs in FP32, so the error is that term's rounding through dt
    (measured 1.6e-7 .. 6.0e-7 for these strongly nonlinear fields; held to 2e-6)."""
    from conftest import smooth_spectral
    from specter_gb300 import api
    plan, g = make_pair(16, 16, 513, 1.0)
    api.set_option(plan, "velocity_split", split)
    rng = np.random.default_rng(40 + solver)
    v = [smooth_spectral(g, rng, amp=0.3) for _ in range(3)]
    th = smooth_spectral(g, rng, amp=0.3)
    pr = g.fftp1d_complex_to_real_z(smooth_spectral(g, rng, amp=1e-3)) / g.nz
    omega = (0.3, -0.7, 2.0) if solver == 2 else (0.0, 0.0, 0.0)
    kw = dict(dt=1e-3, nu=1e-2, ord=2, kappa=5e-3)
    s = api.Solver(plan, solver, fused=True, nl_fp32=True, omega=omega, **kw)
    for fld, a in zip((s.vx, s.vy, s.vz), v):
        fld.upload(a)
    s.pr.upload(pr)
    if solver >= 1:
        s.th.upload(th)
    s.step(2)
    ref = g.run(g.params(**kw), 2, *v, pr, th=th if solver >= 1 else None, omega=omega if solver == 2 else None)
    got = [f.download() for f in (s.vx, s.vy, s.vz)] + ([s.th.download()] if solver >= 1 else [])
    s.close()
    e = [rel(a, b) for a, b in zip(got, ref[: len(got)])]
    print("solver %d split %d: %s" % (solver, split, " ".join("%.2e" % x for x in e)))
    assert max(e) < 2e-6


def test_state_conversions_round_trip():
    """A precision-form solver call converts its FP64 state to float-float and back; with no
    steps the state must come back to 2^-46 relative, zeros as zeros, and magnitudes below the
    float range as (near) zero."""
    from specter_gb300 import api
    plan = api.Plan((16, 16, 58), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 2.0), precision=api.FP64)
    s = api.Solver(plan, api.BOUSS, fused=True, nl_fp32=True, dt=1e-5, nu=1e-4, kappa=1e-4)
    rng = np.random.default_rng(31)
    shape = plan.sshape
    mag = 10.0 ** rng.uniform(-30, 30, shape)
    a = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * mag
    a.flat[::7] = 0.0
    a.flat[3::11] *= 1e-280       # below the float range: the FP64 path
    a.flat[5::13] = -a.flat[5::13]
    fields = (s.vx, s.vy, s.vz, s.th, s.pr)
    for f in fields:
        f.upload(a)
    s.step(0)
    for f in fields:
        b = f.download()
        for x, y in ((a.real, b.real), (a.imag, b.imag)):
            big = np.abs(x) >= 2.0 ** -100
            assert np.all(np.abs(y[big] - x[big]) <= 2.0 ** -46 * np.abs(x[big]))
            assert np.all(np.abs(y[~big]) <= 1e-30)
            assert np.all(y[x == 0] == 0)
    s.close()


def test_nl_fp32_needs_fp64_plan():
    from specter_gb300 import api, SpecterError
    plan = api.Plan((16, 16, 58), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 2.0), precision=api.FP32)
    with pytest.raises(SpecterError) as e:
        api.Solver(plan, api.HD, fused=True, nl_fp32=True)
    assert e.value.code == 7
