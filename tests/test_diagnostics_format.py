"""Fortran 1P Ew.d formatting of the diagnostic writers (CPU)."""
from specter_gb300.diagnostics import BALANCE, NOSLIP, fortran_e, line


def test_fortran_e_fields():
    assert fortran_e(1.0, 13, 6) == " 1.000000E+00"
    assert fortran_e(-2.5e-7, 13, 6) == "-2.500000E-07"
    assert fortran_e(0.0, 23, 16) == " 0.0000000000000000E+00"
    assert fortran_e(123456.789, 13, 6) == " 1.234568E+05"
    assert fortran_e(9.9999995e-3, 13, 6) == " 1.000000E-02"   # rounds up into the next decade
    assert fortran_e(1.5e-100, 13, 6) == " 1.500000-100"       # three-digit exponent drops the E
    assert fortran_e(-1.5e-100, 13, 6) == "-1.500000-100"
    assert fortran_e(-1.5e-100, 12, 6) == "*" * 12             # does not fit the field


def test_line_widths():
    s = line((0.0001, 0.5, 0.25, -1e-3), BALANCE)
    assert len(s) == 13 + 23 + 23 + 24
    assert s.split() == ["1.000000E-04", "5.0000000000000000E-01", "2.5000000000000000E-01", "-1.0000000000000000E-03"]
    assert len(line((1, 2, 3, 4, 5, 6), NOSLIP)) == 6 * 13
