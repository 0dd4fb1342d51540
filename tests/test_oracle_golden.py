"""Pin the C oracle against the committed numpy restatement (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_small.npz")


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


@pytest.fixture(scope="module")
def gold(oracle_mod):
    G = dict(np.load(GOLD))
    nx, ny, nz, cz, oz = (int(x) for x in G["grid"])
    g = oracle_mod.Grid(nx, ny, nz, cz, oz, *G["box"])
    return g, G


def test_transforms(gold):
    g, G = gold
    c = g.fftp3d_real_to_complex(G["r2c_in"])
    assert rel(c, G["r2c_out"]) < 2e-12  # continuation rows amplify rounding ~1e4x (|dir| <= 3.5e3)
    r = g.fftp3d_complex_to_real(G["r2c_out"])
    assert rel(r, G["c2r_out"]) < 2e-12


def test_nonlinear_terms(gold):
    g, G = gold
    v = (G["vx"], G["vy"], G["vz"])
    for got, key in zip(g.gradre(*v), ("gradre_x", "gradre_y", "gradre_z")):
        assert rel(got, G[key]) < 1e-12
    assert rel(g.advect(*v, G["th"]), G["advect"]) < 1e-12
    assert rel(g.fc_filter(G["vx"]), G["filt"]) < 1e-14


def test_projection_and_diagnostics(gold):
    g, G = gold
    v = (G["vx"], G["vy"], G["vz"])
    a, b, c, d = g.sol_project(*v, 1, 0, 0)
    for got, key in zip((a, b, c), ("proj_a", "proj_b", "proj_c")):
        assert rel(got, G[key]) < 1e-12
    nzp = g.nz - g.cz
    assert rel(d[:, :, :nzp], G["proj_d"][:, :, :nzp]) < 1e-12
    assert abs(g.energy(*v, 1) - G["energy1"]) / G["energy1"] < 1e-13
    assert abs(g.energy(*v, 0) - G["energy0"]) / G["energy0"] < 1e-13
    assert abs(g.divergence(*v) - G["divergence"]) / G["divergence"] < 1e-12


def test_rk_steps(gold):
    g, G = gold
    p = g.params(dt=1e-3, nu=1e-2, ord=2, kappa=1e-2)
    vx, vy, vz, pr = g.run(p, 1, G["vx"], G["vy"], G["vz"], G["pr"])
    nzp = g.nz - g.cz
    for got, key in zip((vx, vy, vz), ("hd_vx", "hd_vy", "hd_vz")):
        assert rel(got, G[key]) < 2e-11
    assert rel(pr[:, :, :nzp], G["hd_pr"][:, :, :nzp]) < 2e-11
    vx, vy, vz, th, pr = g.run(p, 1, G["vx"], G["vy"], G["vz"], G["pr"], th=G["th"])
    for got, key in zip((vx, vy, vz, th), ("bo_vx", "bo_vy", "bo_vz", "bo_th")):
        assert rel(got, G[key]) < 2e-11
    assert rel(pr[:, :, :nzp], G["bo_pr"][:, :, :nzp]) < 2e-11
