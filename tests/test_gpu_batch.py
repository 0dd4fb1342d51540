"""Batched ensembles (specter_batch_create), through the C ABI: solvers of uneven grids advanced
by batched launches -- one launch per kernel family and length class for the whole ensemble --
must each end in exactly the state their own solver steps give (same kernel bodies, same
arguments), in a few dozen launches a step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# z lengths 58 / 90 / 122 (Bluestein 128, direct 90, Bluestein 256), x and y lengths 32 ... 96
GRIDS = [(32, 48, 33), (48, 32, 65), (64, 64, 97), (96, 32, 33), (32, 96, 65), (64, 48, 97)]


def _solver(api, initial, nx, ny, nzp, seed, nu):
    plan = api.Plan((nx, ny, nzp + 25), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 2.0), precision=api.FP32)
    api.set_option(plan, "velocity_split", 1)
    s = api.Solver(plan, api.HD, ord=2, dt=1e-4, nu=nu)
    v = initial.channel_velocity(plan, seed=seed, amp=0.05, kmax=8)
    for f, sp in zip((s.vx, s.vy, s.vz), initial.to_spectral(plan, v)):
        f.copy_from(sp)
    s.pr.zero()
    plan.synchronize()
    return plan, s


def test_batch_equals_solo_steps():
    from specter_gb300 import api, initial
    nus = [1e-3, 5e-4, 2e-3, 8e-4, 1.2e-3, 3e-4]
    solo = [_solver(api, initial, *g, seed=11 + i, nu=nus[i]) for i, g in enumerate(GRIDS)]
    bat = [_solver(api, initial, *g, seed=11 + i, nu=nus[i]) for i, g in enumerate(GRIDS)]
    launches0 = sum(p.launch_count for p, _ in solo)
    for _, s in solo:
        s.step(3)
    per_step_solo = (sum(p.launch_count for p, _ in solo) - launches0) / 3
    b = api.Batch([s for _, s in bat])
    b.step(3)
    b.synchronize()
    for (_, x), (_, y) in zip(solo, bat):
        for fx, fy in zip(x.state, y.state):
            assert np.array_equal(fx.download(), fy.download())
    # two stages of seven kernel positions; per position one launch per length class
    assert b.kernels <= 14 * 4 and b.kernels < per_step_solo
    b.close()


def test_batch_rejects_shared_plan_and_fp64():
    from specter_gb300 import api, initial, SpecterError
    plan, s = _solver(api, initial, 32, 32, 33, seed=1, nu=1e-3)
    s2 = api.Solver(plan, api.HD, ord=2, dt=1e-4, nu=1e-3)
    with pytest.raises(SpecterError):
        api.Batch([s, s2])
    p64 = api.Plan((32, 32, 58), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 2.0), precision=api.FP64)
    with pytest.raises(SpecterError):
        api.Batch([api.Solver(p64, api.HD, ord=2, dt=1e-4, nu=1e-3)])
