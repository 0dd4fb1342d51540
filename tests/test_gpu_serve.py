"""The served stream (continuous batching): every result is the same whether the request runs
alone or in the mix, and admission respects the memory budget.

Alone and in the mix the same kernels run on the same data with the same tile widths, so the
results must agree exactly (tolerance 0)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from specter_gb300 import serve
    return serve.draw_requests(5, rate=500.0, seed=99, steps=(12, 30), grid_xy=(32, 48), grid_z=(33, 65))


def _alone(req):
    from specter_gb300 import api, initial, serve
    plan, s = serve.make(api, initial, req, api.FP32)
    s.step(req.steps)
    out = [f.download() for f in s.state]
    s.close()
    plan.close()
    return out


def test_results_same_alone_and_in_mix():
    from specter_gb300 import serve
    reqs = _requests()
    assert {r.kind for r in reqs} == {"HD", "BOUSS"}
    srv = serve.Server(budget_bytes=8e9, chunk=7, keep_results=True, policy="all")
    stats = srv.run(reqs)
    assert stats["peak_running"] >= 2  # requests overlapped on the device
    for r in reqs:
        assert r.done > r.admitted >= 0
        for got, ref in zip(r.result, _alone(r)):
            assert np.array_equal(got, ref), r


def test_budget_admission_serialises():
    from specter_gb300 import serve
    reqs = _requests()
    srv = serve.Server(budget_bytes=1, chunk=50, keep_results=True)
    stats = srv.run(reqs)
    assert stats["peak_active"] == 1
    for r in reqs[:2]:
        for got, ref in zip(r.result, _alone(r)):
            assert np.array_equal(got, ref)


def test_srpt_policy_same_results():
    from specter_gb300 import serve
    reqs = _requests()
    srv = serve.Server(budget_bytes=8e9, chunk=5, keep_results=True, policy="srpt", fill_points=1)
    stats = srv.run(reqs)
    assert stats["peak_running"] == 1 and stats["peak_active"] >= 2  # resident, run one at a time
    for r in reqs:
        for got, ref in zip(r.result, _alone(r)):
            assert np.array_equal(got, ref)
