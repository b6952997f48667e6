"""Fortran input editing of the golden-fixture generator (tests/golden/make_golden.py).

The fixtures hold the reference's input records as the Fortran reads of the
column driver and of rrtatm.f see them: F/E editing with BLANK='NULL',
implied decimals for fields without a point, and one correctly rounded
conversion per field (so '3.20000000e-01' is the double nearest 0.32, not
3.2 * 0.1).  The profile-builder pin depends on that: its layers agree with
the reference's to better than 1e-7.
"""
import importlib.util
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
mg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mg)


@pytest.mark.parametrize("field,d,value", [
    ("   0.32000", 0, 0.32),
    ("3.20000000e-01", 0, 0.32),
    (" 2.09000000e+05", 0, 209000.0),
    ("   -1.5E+2", 0, -150.0),
    ("  1234", 3, 1.234),
    ("  1234", 0, 1234.0),
    ("  12E1", 2, 1.2),
    ("      ", 4, 0.0),
    ("  .5", 0, 0.5),
    ("5.", 0, 5.0),
    (" 1013.0000", 3, 1013.0),
    (" 0.0000611", 3, 6.11e-05),
    ("44.9843", 4, 44.9843),
])
def test_field_values_are_correctly_rounded(field, d, value):
    assert mg.fnum(field, d) == value


def test_bad_field_raises():
    with pytest.raises(ValueError):
        mg.fnum("1.2.3")


def test_fixed_column_record():
    r = mg.Rec("    0    2  -48    1    0    7    1 0  0     0.000   110.000     0.000 0.0000000")
    assert [r.i(5) for _ in range(7)] == [0, 2, -48, 1, 0, 7, 1]
    assert r.i(2) == 0
    r.skip(1)
    assert r.i(2) == 0
    assert [r.f(10, 3) for _ in range(5)] == [0.0, 110.0, 0.0, 0.0, 0.0]
