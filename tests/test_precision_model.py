"""The precision split on the CPU: in the numpy model of the Rayleigh-Benard stage
(tests/golden/precision_model.py), FP32 in an operation that carries the state through a z
transform (the wall round trips, the stored state) puts theta's error orders of magnitude above
what the FP32 nonlinear term alone does -- the reason the nl_fp32 form keeps only the nonlinear
term in FP32."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def test_only_the_nonlinear_term_tolerates_fp32():
    import precision_model as pm
    rows = {r["variant"]: r["rel_l2"] for r in pm.study(8, 10, ["nl=32", "R=32", "state=32"])}
    vx, vy, vz, th = rows["nl=32"]
    assert max(vx, vy, vz) < 2e-6 and th < 1e-10       # measured 7.0e-7, 7.1e-14
    assert max(rows["R=32"]) > 1e-5                     # wall round trips in FP32: 5.7e-5
    assert rows["R=32"][3] > 1e4 * th and rows["state=32"][3] > 1e4 * th   # theta 3.1e-5, 2.2e-6
