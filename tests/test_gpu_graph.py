"""Autotuning and CUDA-graph capture of RK steps (the ensemble form), through the C ABI.

A captured step must give exactly the state that plain solver steps give (same kernels, same
data); the autotuner must leave the state untouched; several solvers of uneven grids captured in
one graph must each advance exactly as they would alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(api, initial, nx, ny, nzp, precision, seed, nu=1e-3):
    plan = api.Plan((nx, ny, nzp + 25), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 2.0), precision=precision)
    s = api.Solver(plan, api.HD, ord=2, dt=1e-4, nu=nu)
    v = initial.channel_velocity(plan, seed=seed, amp=0.05, kmax=8)
    for f, sp in zip((s.vx, s.vy, s.vz), initial.to_spectral(plan, v)):
        f.copy_from(sp)
    s.pr.zero()
    plan.synchronize()
    return plan, s


def _state(s):
    return [f.download() for f in s.state]


GRIDS = [(32, 48, 33), (48, 32, 65), (64, 64, 97)]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_graph_equals_plain_steps(precision):
    from specter_gb300 import api, initial
    plain = [_solver(api, initial, *g, precision, seed=7 + i) for i, g in enumerate(GRIDS)]
    capt = [_solver(api, initial, *g, precision, seed=7 + i) for i, g in enumerate(GRIDS)]
    for _, s in plain:
        s.step(3)
    graph = api.Graph([s for _, s in capt], nsteps=1)
    assert graph.kernels > 0
    for _ in range(3):
        graph.launch()
    graph.synchronize()
    for (_, a), (_, b) in zip(plain, capt):
        for x, y in zip(_state(a), _state(b)):
            assert np.array_equal(x, y)
    graph.close()


def test_autotune_keeps_state_and_results():
    from specter_gb300 import api, initial
    p1, s1 = _solver(api, initial, 48, 48, 65, 1, seed=3)
    p2, s2 = _solver(api, initial, 48, 48, 65, 1, seed=3)
    before = _state(s1)
    caps = s1.autotune()
    assert len(caps) == 5 and all(c in (1, 2, 4, 8, 16) for c in caps[:4]) and caps[4] in (0, 1)
    for x, y in zip(before, _state(s1)):
        assert np.array_equal(x, y)
    # tile widths change the launch shape, not the per-column arithmetic (only the grouping of
    # the FP64 wall sums, whose rounding can move an FP32 result by an ulp)
    api.set_tile_caps(p2, (2, 2, 2, 2))
    s1.step(2)
    s2.step(2)
    for x, y in zip(_state(s1), _state(s2)):
        assert np.allclose(x, y, rtol=0, atol=1e-6 * np.abs(y).max())


def test_graph_query_and_memory():
    from specter_gb300 import api, initial
    _, s = _solver(api, initial, 32, 32, 33, 1, seed=5)
    g = api.Graph([s], nsteps=2)
    g.launch()
    g.synchronize()
    import ctypes as C
    done = C.c_int(-1)
    assert api.load().specter_graph_query(g.h, C.byref(done)) == 0 and done.value == 1
    b = C.c_ulonglong()
    assert api.load().specter_solver_memory(s.h, C.byref(b)) == 0
    assert b.value > 7 * s.plan.nxh * s.plan.ny * s.plan.nz * 8
    g.close()


def test_small_ensemble_run():
    from specter_gb300 import ensemble
    res, insts, built = ensemble.run(instances=4, steps=5, seed=11, seq_sample=2)
    assert res["solves_per_s"] > 0 and res["graph_kernels_per_step"] > 0
    assert res["fp32_vs_fp64_rel_l2_max"] < 1e-5
