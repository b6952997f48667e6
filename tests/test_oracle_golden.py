"""Pin the FP64 oracle against RRTMG_SW's committed example outputs.

The fixtures (tests/golden/std_atm_cases.json, made by make_golden.py) hold
the eleven run_examples_std_atm runs that need no profile builder, with
every printed block: broadband and, for the iout=98 runs, each of the 14
bands.  The reference prints fluxes with 4 decimals (f10.4), net flux with 6
(f11.6) and heating rate with 5 (f10.5) (rrtmg_sw.1col.f90:498-505), so the
tolerance is half a unit in the last printed place plus 1e-9 for the
printing itself.
"""
import json
import os

import numpy as np
import pytest

import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "std_atm_cases.json")))["cases"]
TOL = {"uflx": 5e-5, "difdflx": 5e-5, "dirdflx": 5e-5, "dflx": 5e-5, "fnet": 5e-7, "htr": 5e-6}

PARAMS = []
for c in CASES:
    for b in c["expected"]:
        PARAMS.append(pytest.param(c, b, id="%s-b%d-%d" % (c["name"], b["istart"], b["iend"])))


@pytest.mark.parametrize("case,block", PARAMS)
def test_golden_block(case, block):
    out = pyoracle.column_mode(case, block["istart"], block["iend"], nmca=200)
    for k, tol in TOL.items():
        err = np.max(np.abs(out[k] - np.array(block[k])))
        assert err <= tol + 1e-9, (k, err)


def test_mersenne_twister_known_answer():
    # MT19937 reference output for the standard seed 5489: the 10000th
    # 32-bit output is 4123659995 (C++11 [rand.predef]).
    v = pyoracle.mt_real(5489, 10000)
    assert round(v[-1] * 4294967295.0) == 4123659995


def test_exp_table():
    t = pyoracle.exp_table()
    assert t[0] == 1.0 and t[10000] == 1e-20
    i = np.arange(1, 10000)
    tfn = i / 10000.0
    np.testing.assert_allclose(t[1:10000], np.maximum(np.exp(-(1 / 0.278) * tfn / (1 - tfn)), 1e-20), rtol=1e-15)
