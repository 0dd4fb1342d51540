"""specter_bouncheck_z_static: the no-slip wall check without any allocation.

Some callers may not allocate device memory once they run (a serving loop that has committed
its memory budget, code inside the RK loop that cannot take the synchronisation of
cudaMalloc/cudaFree).  This entry point keeps its working memory in one fixed device array;
here it must reproduce specter_bouncheck_z through the C ABI on consecutive calls (the array
keeps the previous call's contents) and reject grids larger than the array.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(plan, rng):
    shape = plan.sshape
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    b = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    return plan.field(data=a), plan.field(data=b)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_static_matches_allocating(precision):
    from specter_gb300 import api
    plan = api.Plan((32, 24, 58), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 2.0), precision=precision)
    rng = np.random.default_rng(17)
    for call in range(2):  # two calls in a row: the shared array must not leak state
        fa, fb = _fields(plan, rng)
        pair_ref = api.bouncheck_z(plan, fa, fb)
        pair_got = api.bouncheck_z_static(plan, fa, fb)
        assert pair_got == pytest.approx(pair_ref, rel=1e-12, abs=0), call
        one_ref = api.bouncheck_z(plan, fa)
        one_got = api.bouncheck_z_static(plan, fa)
        assert one_got == pytest.approx(one_ref, rel=1e-12, abs=0), call


def test_static_rejects_large_grid():
    from specter_gb300 import api, SpecterError
    plan = api.Plan((512, 512, 58), (0, 0, 25), (0, 0, 5), (1.0, 1.0, 1.0), precision=1)
    f = plan.field()
    with pytest.raises(SpecterError) as e:
        api.bouncheck_z_static(plan, f)
    assert e.value.code == 1
