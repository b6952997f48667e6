"""Per-band fluxes (the band loop of rrtmg_sw_spcvmc.f90:619-630 that the
column driver prints with iout = 98).

CPU: in the oracle the bands add up to the broadband fluxes.  GPU: the
library's band fluxes against the oracle's, FP64 form to 1e-9 relative element by element, and
their sum against its own broadband fluxes.
"""
import numpy as np
import pytest

import pyoracle
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

BANDS = ("bndfu", "bndfd", "bndfddir", "bndcu", "bndcd")
BROAD = {"bndfu": "swuflx", "bndfd": "swdflx", "bndcu": "swuflxc", "bndcd": "swdflxc"}


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    pyoracle.init(1.004e3)


def case(ncol=24, nlay=47, seed=41):
    c = make_columns(ncol, nlay, seed, clouds=True, aerosol=True)
    m = pyoracle.mcica_subcol_sw(ncol, nlay, 2, 112, 0, *(c[k].ravel(order="F") for k in
                                                         ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                 np.zeros(14 * ncol * nlay), np.ones(14 * ncol * nlay), np.zeros(14 * ncol * nlay),
                                 np.zeros(14 * ncol * nlay), np.zeros(ncol * nlay))
    names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
    shp = {k: (112, ncol, nlay) for k in names}
    shp.update(reicmcl=(ncol, nlay), relqmcl=(ncol, nlay))
    mc = tuple(m[k].reshape(shp[k], order="F") for k in names)
    return gcm_inputs(c, icld=2, iaer=10, mcica=mc)


def oracle_bands(kw):
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS}
    for k in pyoracle.MCICA_INPUTS + pyoracle.AER_INPUTS:
        if kw.get(k) is not None:
            inp[k] = kw[k]
    out = pyoracle.rrtmg_sw(kw["ncol"], kw["nlay"], kw["icld"], kw["iaer"], inp, bands=True)
    ncol, nlay = kw["ncol"], kw["nlay"]
    res = {k: out[k].reshape((ncol, nlay + 1, 14), order="F") for k in BANDS}
    res.update({k: out[k].reshape((ncol, nlay + 1), order="F") for k in BROAD.values()})
    return res


def test_oracle_bands_sum_to_broadband():
    o = oracle_bands(case())
    for b, f in BROAD.items():
        np.testing.assert_allclose(o[b].sum(axis=2), o[f], rtol=1e-12, atol=1e-9, err_msg=b)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_gpu_bands(form):
    from rrtmg_sw_gb300 import build, interface as gpu
    build.build()
    gpu.rrtmg_sw_ini(1.004e3)
    gpu.set_form(gpu.FORM_FP64 if form == "fp64" else gpu.FORM_FP32)
    try:
        kw = case()
        g = gpu.rrtmg_sw(**kw, bands=True)
    finally:
        gpu.set_form(gpu.FORM_FP64)
    o = oracle_bands(kw)
    for k in BANDS:
        if form == "fp64":
            # every element within 1e-9 relative, floor 1e-9 W m-2 near zero
            d = np.abs(g[k] - o[k])
            bad = d > 1e-9 * np.abs(o[k]) + 1e-9
            assert not bad.any(), (k, int(bad.sum()), float(np.max(d)))
        else:
            assert np.max(np.abs(g[k] - o[k])) <= 0.05, k
    for b, f in BROAD.items():
        np.testing.assert_allclose(g[b].sum(axis=2), g[f], rtol=1e-5, atol=2e-3, err_msg=b)
