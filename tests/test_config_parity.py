"""GPU library vs the FP64 oracle at the benchmark configurations' own
sizes, element by element, with the discrete choices checked directly.

* Clear sky, 1024 columns x 60 layers, FP64 form (the plain-method clear-sky
  configuration): every flux and heating rate within |d| <= 1e-9 |ref| +
  floor (floors 1e-9 W m-2 and 1e-8 K/day, for values near zero), and the
  setcoef_sw indices jp, jt, jt1, indself, indfor and laytrop identical for
  every column and layer (rrtmg_sw_setcoef.f90:158-200).
* setcoef_sw's indices at their boundaries (pressures on the jp grid and at
  the laytrop threshold, temperatures on the indself / indfor grids, moved by
  up to 3e-7 relative): identical to the oracle's in both arithmetic forms.
* McICA clouds (icld=2, inflgsw=2 iceflgsw=3 liqflgsw=1) with aerosol
  (iaer=10), 16384 columns x 60 layers, FP64 form: the seven subcolumn arrays
  of mcica_subcol_sw identical to the oracle's for all 16384 columns, and the
  fused solve within the same elementwise bound.  Both are compared in chunks
  of 2048 columns (KISS subcolumn streams are per column, so chunks give the
  call's values) to bound host memory.
* Cloud-optics branches no example run exercises: ice flags 1 and 2
  (rrtmg_sw_cldprmc.f90:182-234) and inflgsw=0, cloud optical properties
  given directly (:150-163): FP64 form at the same bound, FP32 form within
  0.05 W m-2 and 0.01 K/day.

Seeds follow the benchmark configurations: 20261203 + configuration index.
"""
import numpy as np
import pytest

import pyoracle
from rrtmg_sw_gb300 import interface as gpu
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

pytestmark = pytest.mark.gpu

FLUX = ("swuflx", "swdflx", "swuflxc", "swdflxc")
HR = ("swhr", "swhrc")
MC_NAMES = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")


@pytest.fixture(scope="module", autouse=True)
def _init():
    from rrtmg_sw_gb300 import build
    build.build()
    gpu.rrtmg_sw_ini(1.004e3)
    pyoracle.init(1.004e3)
    yield
    gpu.set_form(gpu.FORM_FP64)


def assert_elementwise(g, o, rtol=1e-9, flux_floor=1e-9, hr_floor=1e-8):
    for keys, floor in ((FLUX, flux_floor), (HR, hr_floor)):
        for k in keys:
            d = np.abs(g[k] - o[k])
            lim = rtol * np.abs(o[k]) + floor
            bad = d > lim
            assert not bad.any(), (k, int(bad.sum()), float(np.max(d / (np.abs(o[k]) + 1e-300))))


def oracle_solve(kw):
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS}
    for k in pyoracle.MCICA_INPUTS + pyoracle.AER_INPUTS:
        if kw.get(k) is not None:
            inp[k] = kw[k]
    out = pyoracle.rrtmg_sw(kw["ncol"], kw["nlay"], kw["icld"], kw["iaer"], inp, inflgsw=kw["inflgsw"],
                            iceflgsw=kw["iceflgsw"], liqflgsw=kw["liqflgsw"])
    ncol, nlay = kw["ncol"], kw["nlay"]
    return {k: v.reshape((ncol, nlay if k in HR else nlay + 1), order="F") for k, v in out.items() if k in FLUX + HR}


def gpu_solve(kw, clouds=None):
    res = gpu.rrtmg_sw(**kw, clouds=clouds, extra=True)
    return {k: res[k] for k in FLUX + HR}


def sub(c, lo, hi):
    """Columns lo:hi of a make_columns dict."""
    return {k: (v[lo:hi] if isinstance(v, np.ndarray) and v.shape[:1] == (c["play"].shape[0],) else v)
            for k, v in c.items()}


def oracle_mcica(c, icld, seed, tauc=None, ssac=None, asmc=None, fsfc=None):
    ncol, nlay = c["play"].shape
    z14 = np.zeros(14 * ncol * nlay)
    f = lambda x, d: d if x is None else np.asarray(x).ravel(order="F")
    m = pyoracle.mcica_subcol_sw(ncol, nlay, icld, seed, 0, *(c[k].ravel(order="F") for k in
                                                              ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                 f(tauc, z14), f(ssac, z14 + 1.0), f(asmc, z14), f(fsfc, z14), np.zeros(ncol * nlay))
    shp = {k: (112, ncol, nlay) for k in MC_NAMES}
    shp.update(reicmcl=(ncol, nlay), relqmcl=(ncol, nlay))
    return tuple(m[k].reshape(shp[k], order="F") for k in MC_NAMES)


def test_clear_sky_1024x60_fp64_elementwise_and_indices():
    c = make_columns(1024, 60, 20261203 + 0)
    kw = gcm_inputs(c, icld=0, iaer=0)
    assert_elementwise(gpu_solve(kw), oracle_solve(kw))
    g = gpu.setcoef_indices(**kw)
    o = pyoracle.gcm_setcoef_indices(kw)
    for k in ("jp", "jt", "jt1", "indself", "indfor", "laytrop"):
        np.testing.assert_array_equal(g[k], o[k], err_msg=k)
    assert g["jp"].min() >= 1 and g["jp"].max() <= 58 and g["laytrop"].min() >= 1


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_setcoef_indices_at_their_boundaries(form):
    # pressures on the jp grid (36 - 5 (ln p + 0.04) integer) and at the
    # laytrop threshold ln p = 4.56, temperatures on the indself / indfor
    # grids, each moved by 0, +-1e-7 or +-3e-7 relative: both forms return the
    # FP64 indices (the FP32 form re-evaluates near-integer values in FP64)
    ncol, nlay = 2048, 60
    c = make_columns(ncol, nlay, 20261277)
    rng = np.random.default_rng(20261278)
    dl = np.array([-3e-7, -1e-7, 0.0, 1e-7, 3e-7])
    grid = np.concatenate([np.exp((36.0 - np.arange(1, 59)) / 5.0 - 0.04), [np.exp(4.56)]])
    p = np.sort(rng.choice(grid, (ncol, nlay)), axis=1)[:, ::-1] * (1.0 + rng.choice(dl, (ncol, nlay)))
    tgrid = np.concatenate([188.0 + 7.2 * np.arange(8, 17), 332.0 - 36.0 * np.arange(1, 3)])
    t = rng.choice(tgrid, (ncol, nlay)) * (1.0 + rng.choice(dl, (ncol, nlay)))
    kw = gcm_inputs(c, icld=0, iaer=0)
    kw["play"], kw["tlay"] = p, t
    gpu.set_form(gpu.FORM_FP32 if form == "fp32" else gpu.FORM_FP64)
    try:
        g = gpu.setcoef_indices(**kw)
    finally:
        gpu.set_form(gpu.FORM_FP64)
    o = pyoracle.gcm_setcoef_indices(kw)
    for k in ("jp", "jt", "jt1", "indself", "indfor", "laytrop"):
        np.testing.assert_array_equal(g[k], o[k], err_msg=k)


def test_mcica_aerosol_16384x60_fp64_masks_and_fluxes():
    ncol, nlay, chunk = 16384, 60, 2048
    c = make_columns(ncol, nlay, 20261203 + 1, clouds=True, aerosol=True)
    z = np.zeros((14, chunk, nlay))
    for lo in range(0, ncol, chunk):
        cc = sub(c, lo, lo + chunk)
        o = oracle_mcica(cc, 2, 112)
        g = gpu.mcica_subcol_sw(1, chunk, nlay, 2, 112, 0, cc["play"], cc["cldfrac"], cc["ciwp"], cc["clwp"],
                                cc["rei"], cc["rel"], z, z + 1.0, z, z, None)
        for name, a, b in zip(MC_NAMES, g, o):
            np.testing.assert_array_equal(a, b, err_msg="%s columns %d.." % (name, lo))
        # the fused solve of the chunk against the oracle on those subcolumns
        kwo = gcm_inputs(cc, icld=2, iaer=10, mcica=o)
        clouds = dict(permuteseed=112, irng=0, cldfrac=cc["cldfrac"], ciwp=cc["ciwp"], clwp=cc["clwp"],
                      rei=cc["rei"], rel=cc["rel"])
        assert_elementwise(gpu_solve(gcm_inputs(cc, icld=2, iaer=10), clouds), oracle_solve(kwo))


@pytest.mark.parametrize("inflg,iceflg", [(2, 1), (2, 2), (0, 3)])
def test_cloud_optics_branches(inflg, iceflg):
    ncol, nlay = 256, 60
    c = make_columns(ncol, nlay, 20261240 + 3 * inflg + iceflg, clouds=True)
    tauc = ssac = asmc = fsfc = None
    if inflg == 0:
        # cloud optical properties given per band (cldprmc.f90:150-163)
        rng = np.random.default_rng(11)
        cloudy = (c["cldfrac"] > 0)[None, :, :]
        tauc = np.where(cloudy, rng.uniform(0.5, 30.0, (14, ncol, nlay)), 0.0)
        ssac = rng.uniform(0.85, 0.9999, (14, ncol, nlay))
        asmc = rng.uniform(0.7, 0.9, (14, ncol, nlay))
        fsfc = asmc ** 2
    o_mc = oracle_mcica(c, 2, 112, tauc, ssac, asmc, fsfc)
    kwo = gcm_inputs(c, icld=2, iaer=0, mcica=o_mc)
    kwo.update(inflgsw=inflg, iceflgsw=iceflg)
    ref = oracle_solve(kwo)
    kwf = gcm_inputs(c, icld=2, iaer=0)
    kwf.update(inflgsw=inflg, iceflgsw=iceflg)
    clouds = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
                  rel=c["rel"], tauc=tauc, ssac=ssac, asmc=asmc, fsfc=fsfc)
    assert_elementwise(gpu_solve(kwf, clouds), ref)
    gpu.set_form(gpu.FORM_FP32)
    try:
        g32 = gpu_solve(kwf, clouds)
    finally:
        gpu.set_form(gpu.FORM_FP64)
    for k in FLUX:
        assert np.max(np.abs(g32[k] - ref[k])) <= 0.05, (k, float(np.max(np.abs(g32[k] - ref[k]))))
    for k in HR:
        assert np.max(np.abs(g32[k] - ref[k])) <= 0.01, (k, float(np.max(np.abs(g32[k] - ref[k]))))
