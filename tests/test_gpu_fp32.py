"""FP32-bulk (precision form) kernels against the FP64 oracle on grids that select the
register four-step FFT kernels: 256 x 256 x 257 (+25) -> y 256 = 16*16, x H = 128 = 16*8,
z Bluestein 576 = 24*24; 128 x 128 x 513 (+25) -> z Bluestein 1080 = 36*30; and the small
grids of the ensemble and the served stream: z 90 = 10*9 directly, Bluestein 128 = 16*8 (nz 58),
256 = 16*16 (nz 122), 320 = 20*16 (nz 154); x H = 16 ... 64 and y 32 ... 128 (SPLITS below).

FP32 rounding of the d wall-adjacent points is amplified by the continuation (sum |dir| = 9.5e3):
rounding a smooth column to FP32 alone (2.5e-8) already gives ~2e-5 relative error in its
continued spectrum (tests/test_fc_conditioning.py), so transforms through the continuation are
held to 3e-4 against the FP64 oracle and C2R (no continuation) to 1e-6; one RK2 step to about 3x
the largest error measured on these grids (fused velocity 1e-4, theta 1.5e-3).  This form does
not meet 1e-5 after 1000 steps (its errors grow with the step count); the precision form that
does is tests/test_gpu_precision.py."""
import numpy as np
import pytest

from conftest import make_pair, rel, smooth_spectral

pytestmark = pytest.mark.gpu


def smooth_real(g, rng, nmodes=6, kmax=4):
    x = 2 * np.pi * np.arange(g.nx) / g.nx
    y = 2 * np.pi * np.arange(g.ny) / g.ny
    Z, Y, X = np.meshgrid(g.z, y, x, indexing="ij")
    r = np.zeros(g.rshape)
    for _ in range(nmodes):
        kx, ky = rng.integers(-kmax, kmax + 1, 2)
        r += rng.standard_normal() * np.cos(kx * X + ky * Y + rng.uniform(0.3, 4.0) * Z + rng.uniform(0, 6.3))
    r[g.nz - g.cz:] = 0
    return r


# grid -> expected engine per axis: (L, L1, L2, Bluestein)
SPLITS = {
    (256, 256, 257): {"x": (128, 16, 8, False), "y": (256, 16, 16, False), "z": (576, 24, 24, True)},
    (128, 128, 513): {"x": (64, 8, 8, False), "y": (128, 16, 8, False), "z": (1080, 36, 30, True)},
    (48, 96, 65): {"x": (24, 6, 4, False), "y": (96, 12, 8, False), "z": (90, 10, 9, False)},
    (32, 64, 33): {"x": (16, 4, 4, False), "y": (64, 8, 8, False), "z": (128, 16, 8, True)},
    (64, 48, 97): {"x": (32, 8, 4, False), "y": (48, 8, 6, False), "z": (256, 16, 16, True)},
    (96, 32, 129): {"x": (48, 8, 6, False), "y": (32, 8, 4, False), "z": (320, 20, 16, True)},
}
GRIDS = [(256, 256, 257, 2.0), (128, 128, 513, 1.0), (48, 96, 65, 2.0), (32, 64, 33, 2.0), (64, 48, 97, 2.0),
         (96, 32, 129, 2.0)]


@pytest.fixture(scope="module", params=GRIDS, ids=["256", "128x513", "48x96x65", "32x64x33", "64x48x97", "96x32x129"])
def pair32(request):
    nx, ny, nzp, Lz = request.param
    return make_pair(nx, ny, nzp, Lz, precision=1)


def test_engine_splits(pair32):
    """Each grid runs the four-step split it is meant to exercise (not the generic engine)."""
    plan, g = pair32
    want = SPLITS[(plan.nx, plan.ny, plan.nzp)]
    for ax in "xyz":
        e = plan.engines[ax]
        assert (e["L"], e["L1"], e["L2"], e["bluestein"]) == want[ax], (ax, e)


def test_transforms_fp32(pair32):
    from specter_gb300 import api
    plan, g = pair32
    rng = np.random.default_rng(11)
    r = smooth_real(g, rng)
    out = plan.field()
    api.fftp3d_real_to_complex(plan, plan.field(1, data=r), out)
    ref = g.fftp3d_real_to_complex(r)
    e1 = rel(out.download(), ref)
    rout = plan.field(1)
    api.fftp3d_complex_to_real(plan, plan.field(data=ref), rout)
    e2 = rel(rout.download(), g.fftp3d_complex_to_real(ref))
    print(f"r2c {e1:.2e} c2r {e2:.2e}")
    assert e1 < 3e-4 and e2 < 1e-6


def test_nonlinear_fp32(pair32):
    from specter_gb300 import api
    plan, g = pair32
    rng = np.random.default_rng(12)
    v = [smooth_spectral(g, rng) for _ in range(3)]
    th = smooth_spectral(g, rng)
    fv = [plan.field(data=x) for x in v]
    out = [plan.field() for _ in range(3)]
    api.gradre(plan, *fv, *out)
    errs = [rel(o.download(), r) for o, r in zip(out, g.gradre(*v))]
    fe = plan.field()
    api.advect(plan, *fv, plan.field(data=th), fe)
    errs.append(rel(fe.download(), g.advect(*v, th)))
    print("nonlinear", ["%.2e" % e for e in errs])
    assert max(errs) < 1e-3


def test_projection_fp32(pair32):
    from specter_gb300 import api
    plan, g = pair32
    rng = np.random.default_rng(13)
    v = [smooth_spectral(g, rng) for _ in range(3)]
    pr = g.fftp1d_complex_to_real_z(smooth_spectral(g, rng, amp=1e-2)) / g.nz
    f = [plan.field(data=x) for x in v]
    fp = plan.field(data=pr)
    api.v_imposebc_and_project(plan, *f, fp, 1, 2)
    ref = g.v_imposebc_and_project(*v, pr, 1, 2)
    errs = [rel(a.download(), b) for a, b in zip(f, ref[:3])]
    print("projection", ["%.2e" % e for e in errs])
    assert max(errs) < 5e-4


@pytest.mark.parametrize("solver", [0, 1], ids=["HD", "BOUSS"])
def test_stage_fp32(pair32, solver):
    """One RK2 step of the FP32 form, both the reference call sequence and the fused kernels,
    against the FP64 oracle; the two FP32 paths against each other."""
    from specter_gb300 import api
    plan, g = pair32
    rng = np.random.default_rng(14 + solver)
    v = [smooth_spectral(g, rng, amp=0.3) for _ in range(3)]
    th = smooth_spectral(g, rng, amp=0.3)
    pr = np.zeros(g.sshape, complex)
    kw = dict(dt=1e-4, nu=1e-3, ord=2, kappa=1e-3)
    ref = g.run(g.params(**kw), 1, *v, pr, th=th if solver == 1 else None)
    outs = {}
    for fused in (False, True):
        s = api.Solver(plan, solver, fused=fused, **kw)
        for fld, a in zip((s.vx, s.vy, s.vz), v):
            fld.upload(a)
        if solver == 1:
            s.th.upload(th)
        s.step(1)
        outs[fused] = [f.download() for f in (s.vx, s.vy, s.vz)] + ([s.th.download()] if solver == 1 else [])
        errs = [rel(a, b) for a, b in zip(outs[fused], ref[: len(outs[fused])])]
        print("stage fused=%s" % fused, ["%.2e" % e for e in errs])
        # about 3x the largest error measured over the six grids: fused velocity 3.3e-5, reference
        # sequence velocity 3.0e-4 (its z component goes through two more FP32 continuations),
        # theta (both paths) 4.2e-4
        assert max(errs[:3]) < (1e-4 if fused else 1e-3)
        if solver == 1:
            assert errs[3] < 1.5e-3
    cons = [rel(a, b) for a, b in zip(outs[True], outs[False])]
    print("fused vs reference sequence", ["%.2e" % e for e in cons])
    assert max(cons) < 1e-3


@pytest.mark.parametrize("shape", [(256, 32, 33), (512, 16, 33)], ids=["H128", "H256"])
def test_x_pass_eight_rows(shape):
    """At 8 rows (the autotuned width of the headline grid) the nonlinear x pass of H = 128 and 256
    runs the copy compiled with the row count fixed; at 16 rows the runtime-width copy.  Both
    against the oracle and each other, and a full fused RK2 stage at 8 rows against the oracle."""
    from specter_gb300 import api
    nx, ny, nzp = shape
    plan, g = make_pair(nx, ny, nzp, 2.0, precision=1)
    rng = np.random.default_rng(16)
    v = [smooth_spectral(g, rng) for _ in range(3)]
    th = smooth_spectral(g, rng)
    ref_nl = g.gradre(*v)
    ref_th = g.advect(*v, th)
    got = {}
    for cap in (8, 16):
        api.set_tile_caps(plan, [16, 16, cap, 16])
        nl = [plan.field() for _ in range(3)]
        fv = [plan.field(data=x) for x in v]
        api.gradre(plan, *fv, *nl)
        fe = plan.field()
        api.advect(plan, *fv, plan.field(data=th), fe)
        got[cap] = [f.download() for f in nl] + [fe.download()]
        errs = [rel(a, b) for a, b in zip(got[cap], list(ref_nl) + [ref_th])]
        print(cap, ["%.2e" % e for e in errs])
        assert max(errs) < 1e-3
    cross = [rel(a, b) for a, b in zip(got[8], got[16])]
    print("rows 8 vs 16", ["%.2e" % e for e in cross])
    assert max(cross) < 1e-3
    # one fused BOUSS RK2 step with the 8-row x pass
    api.set_tile_caps(plan, [16, 16, 8, 16])
    kw = dict(dt=1e-4, nu=1e-3, ord=2, kappa=1e-3)
    pr = np.zeros(g.sshape, complex)
    ref = g.run(g.params(**kw), 1, *v, pr, th=th)
    s = api.Solver(plan, 1, fused=True, **kw)
    for fld, x in zip((s.vx, s.vy, s.vz), v):
        fld.upload(x)
    s.th.upload(th)
    s.step(1)
    errs = [rel(f.download(), r) for f, r in zip((s.vx, s.vy, s.vz, s.th), ref[:4])]
    print("stage", ["%.2e" % e for e in errs])
    assert max(errs[:3]) < 1e-4 and errs[3] < 1e-3  # measured: velocity <= 2.4e-5, theta 2.8e-4
