"""CPU-only checks of the C ABI library: it builds, loads, and exports every
entry point declared in include/rrtmg_sw_gb300.h (no compute calls)."""
import ctypes
import os
import re

import numpy as np

from rrtmg_sw_gb300 import build, interface
from rrtmg_sw_gb300.synthetic import make_columns

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rrtmg_sw_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*\**\s*(\w+_c)\s*\(", text)))


def test_library_exports_all_declared_symbols():
    build.build()
    lib = ctypes.CDLL(interface.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


def test_struct_layout_matches_header_field_count():
    text = open(os.path.join(ROOT, "include", "rrtmg_sw_gb300.h")).read()
    body = text[text.index("typedef struct rrtmg_sw_args"):text.index("} rrtmg_sw_args;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    decls = [d for d in body.split(";")[:-1]]
    n = 0
    for d in decls:
        d = d.split("{", 1)[-1]
        n += len([x for x in d.split(",") if x.strip()])
    assert n == len(interface.RrtmgSwArgs._fields_)


def test_errstr_without_gpu():
    build.build()
    lib = interface.lib()
    assert lib.rrtmg_sw_errstr_c(12).decode() == "ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS"
    assert lib.rrtmg_sw_errstr_c(21).decode().startswith("MCICA_SUBCOL: KISSVEC SEED GENERATOR")


def test_synthetic_columns_are_monotonic_and_bounded():
    c = make_columns(200, 60, 20261203, clouds=True, aerosol=True)
    assert np.all(np.diff(c["plev"], axis=1) < 0)
    assert np.all(c["play"] < c["plev"][:, :-1]) and np.all(c["play"] > c["plev"][:, 1:])
    assert c["h2ovmr"].min() >= 3e-6
    assert 0.1 <= c["cldfrac"][c["cldfrac"] > 0].min() and c["cldfrac"].max() <= 1.0
    assert c["rei"].min() >= 5.0 and c["rei"].max() <= 140.0
    assert c["rel"].min() >= 2.5 and c["rel"].max() <= 60.0
