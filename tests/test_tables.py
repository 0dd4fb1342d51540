"""FC-Gram table validation (specter_table_check, no GPU): orthonormal Gram basis and the
continuation's amplification for the packaged C = 25, d = 5 tables; broken tables are reported."""
import os

import numpy as np
import pytest


def test_packaged_tables():
    from specter_gb300 import api
    e, mx, rs = api.table_check(25, 5)
    assert e < 1e-13                      # Q^T Q = I
    assert 3.0e3 < mx < 4.0e3             # |dir| max ~ 3.5e3
    assert 9.0e3 < rs < 1.0e4             # row sums ~ 9.5e3


def test_broken_and_missing_tables(tmp_path):
    from specter_gb300 import api, SpecterError
    A = np.fromfile(os.path.join(api.TABLES, "A25-5.dat"))
    Q = np.fromfile(os.path.join(api.TABLES, "Q5.dat")).reshape(5, 5, order="F")
    A.tofile(tmp_path / "A25-5.dat")
    Qb = Q.copy()
    Qb[0, 0] *= 1.01
    Qb.ravel(order="F").tofile(tmp_path / "Q5.dat")
    e, _, _ = api.table_check(25, 5, str(tmp_path))
    assert e > 1e-3
    with pytest.raises(SpecterError) as err:
        api.table_check(27, 5, str(tmp_path))
    assert err.value.code == 2           # SPECTER_ERR_TABLE
    (tmp_path / "Q4.dat").write_bytes(b"\\0" * 8)
    with pytest.raises(SpecterError):
        api.table_check(25, 4, str(tmp_path))
