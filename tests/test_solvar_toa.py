"""Solar variability (isolvar 0-3) pinned at the top of the atmosphere.

The five iatm = 1 example runs take their layers from the profile builder
rrtatm.f; their full tables are reproduced from the oracle's restatement of
that builder (test_rrtatm_golden.py, and test_gcm_golden.py through the GPU
library).  This test isolates the solar-variability settings where the
tables do not depend on the layers, the top-of-atmosphere rows: the
downward flux there is the band's solar source times cos(sza)
(rrtmg_sw_spcvmc.f90:349-356, the taumol ssi terms, e.g.
rrtmg_sw_taumol.f90:364-378), with the facular, sunspot and
quiet-sun factors of the solar-variability options (rrtmg_sw_rad.f90:
1327-1496).  Bands 16, 20, 23, 25, 26, 27 and 29 take their source without
interpolation in a gas ratio, so their rows do not depend on the layers at
all; the other bands interpolate at the reference layer, and the seeded
mid-latitude column used here reproduces them as well.  Tolerance: half a
unit in the printed 4th decimal (f10.4) plus 1e-9 (FP64 form and oracle);
1e-3 W m-2 for the FP32 form.

Each case passes the column driver's solar record to the GCM interface as
the driver does (rrtmg_sw.1col.f90:1391-1436): solvar(16:17) become
indsolvar for isolvar 1 and 2, solvar(16:29) become bndsolvar for isolvar
3, and solcycfrac is passed for isolvar 1.
"""
import json
import os

import numpy as np
import pytest

import pyoracle
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "solvar_toa_cases.json")))["cases"]
TOL = 5e-5 + 1e-9
NLAY = 60


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    pyoracle.init(1.004e3)


def solar_args(case):
    iso, sv = case["isolvar"], case["solvar"]
    kw = dict(adjes=1.0, dyofyr=case["juldat"], scon=case["scon"], isolvar=iso)
    if iso in (1, 2):
        kw["indsolvar"] = np.array(sv[:2])
    if iso == 1:
        kw["solcycfrac"] = np.array([case["solcycfrac"]])
    if iso in (-1, 3):
        kw["bndsolvar"] = np.array(sv)
    return kw


def column(case):
    c = make_columns(1, NLAY, 5, clouds=False)
    kw = gcm_inputs(c, icld=0, iaer=0)
    kw["coszen"] = np.array([case["zenith"]])
    for k in ("asdir", "asdif", "aldir", "aldif"):
        kw[k] = np.array([case["albedo"][0]])
    return kw


def check(case, swdflx, bndfd, bndfddir, tol=TOL):
    for t in case["toa"]:
        if t["istart"] == t["iend"]:
            ib = t["istart"] - 16
            got, gdir = bndfd[0, -1, ib], bndfddir[0, -1, ib]
        else:
            got, gdir = swdflx[0, -1], None
        assert abs(got - t["dflx"]) <= tol, (case["name"], t["istart"], t["iend"], got, t["dflx"])
        if gdir is not None:
            assert abs(gdir - t["dirdflx"]) <= tol, (case["name"], t["istart"], gdir, t["dirdflx"])


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_solar_variability_toa(case):
    kw = column(case)
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS}
    out = pyoracle.rrtmg_sw(1, NLAY, 0, 0, inp, bands=True, **solar_args(case))
    shp = (1, NLAY + 1, 14)
    check(case, out["swdflx"].reshape((1, NLAY + 1), order="F"), out["bndfd"].reshape(shp, order="F"),
          out["bndfddir"].reshape(shp, order="F"))


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_gpu_solar_variability_toa(form):
    from rrtmg_sw_gb300 import build, interface as gpu
    build.build()
    gpu.rrtmg_sw_ini(1.004e3)
    gpu.set_form(gpu.FORM_FP64 if form == "fp64" else gpu.FORM_FP32)
    try:
        for case in CASES:
            kw = column(case)
            kw.update(solar_args(case))
            g = gpu.rrtmg_sw(**kw, bands=True)
            # FP32 form: its g-point sums carry ~1e-7 relative rounding (1e-4 of 960 W m-2)
            check(case, g["swdflx"], g["bndfd"], g["bndfddir"], TOL if form == "fp64" else 1e-3)
    finally:
        gpu.set_form(gpu.FORM_FP64)
