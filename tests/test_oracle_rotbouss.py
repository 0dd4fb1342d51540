"""The oracle's ROTBOUSS stage (rotbouss_rkstep2.f90) against its BOUSS stage (bouss_rkstep2.f90).

With omega = 0 the two stage bodies differ only in the scalar's tail: BOUSS filters theta and
passes it through c2r -> /(nx ny nz) -> r2c after s_imposebc (bouss_rkstep2.f90:54-59), ROTBOUSS
stops after s_imposebc.  So one stage gives identical velocity and pressure, and BOUSS's theta
is that tail applied to ROTBOUSS's theta.  With omega != 0 the velocity changes, theta's
update (which does not see the Coriolis term) does not."""
import numpy as np

from conftest import rel, smooth_spectral


def test_rotbouss_stage_structure(oracle_mod):
    g = oracle_mod.Grid(16, 12, 33 + 25, 25, 5, 1.0, 1.0, 1.0)
    rng = np.random.default_rng(21)
    v = [smooth_spectral(g, rng, amp=0.3) for _ in range(3)]
    th = smooth_spectral(g, rng, amp=0.3)
    pr = g.fftp1d_complex_to_real_z(smooth_spectral(g, rng, amp=1e-3)) / g.nz
    p = g.params(dt=1e-3, nu=1e-2, ord=2, kappa=5e-3)
    C = [x.copy() for x in v] + [th.copy()]
    b = g.bouss_stage(p, 2, *v, th, pr, *C)
    r = g.rotbouss_stage(p, (0.0, 0.0, 0.0), 2, *v, th, pr, *C)
    for i in (0, 1, 2, 4):
        assert np.array_equal(b[i], r[i])
    tail = g.fftp3d_real_to_complex(g.fftp3d_complex_to_real(g.fc_filter(r[3])) / (g.nx * g.ny * g.nz))
    assert rel(b[3], tail) < 1e-13
    w = g.rotbouss_stage(p, (0.3, -0.7, 2.0), 2, *v, th, pr, *C)
    assert np.array_equal(w[3], r[3])
    assert rel(w[0], r[0]) > 1e-6
