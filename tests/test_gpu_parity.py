"""GPU library vs the FP64 oracle on the same seeded inputs.

Tolerances (stated per test): the plain FP64 form must match the oracle
element by element, |d| <= 1e-9 |ref| + floor, with floors of 1e-9 W m-2 on
fluxes and 1e-8 K/day on heating rates for values near zero (night
columns, the top layers); McICA masks and subcolumn arrays must be
bit-exact; the FP32 form must stay within 0.05 W m-2 on fluxes and
0.01 K/day on heating rates.
"""
import numpy as np
import pytest

import pyoracle
from rrtmg_sw_gb300 import interface as gpu
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

pytestmark = pytest.mark.gpu

FLUX = ("swuflx", "swdflx", "swuflxc", "swdflxc")
HR = ("swhr", "swhrc")


@pytest.fixture(scope="module", autouse=True)
def _init():
    from rrtmg_sw_gb300 import build
    build.build()
    gpu.rrtmg_sw_ini(1.004e3)
    pyoracle.init(1.004e3)
    yield
    gpu.set_form(gpu.FORM_FP64)


def oracle_call(kw, extra=False, idelm=1):
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS}
    for k in pyoracle.MCICA_INPUTS + pyoracle.AER_INPUTS:
        if kw.get(k) is not None:
            inp[k] = kw[k]
    out = pyoracle.rrtmg_sw(kw["ncol"], kw["nlay"], kw["icld"], kw["iaer"], inp, adjes=kw["adjes"],
                            dyofyr=kw["dyofyr"], scon=kw["scon"], isolvar=kw["isolvar"], inflgsw=kw["inflgsw"],
                            iceflgsw=kw["iceflgsw"], liqflgsw=kw["liqflgsw"], idelm=idelm, extra=extra)
    ncol, nlay = kw["ncol"], kw["nlay"]
    shp = {k: (ncol, nlay + 1) for k in out}
    shp.update(swhr=(ncol, nlay), swhrc=(ncol, nlay))
    return {k: v.reshape(shp[k], order="F") for k, v in out.items()}


def gpu_call(kw, extra=False, idelm=1, clouds=None):
    args = dict(kw)
    res = gpu.rrtmg_sw(**args, idelm=idelm, extra=True, clouds=clouds)
    return res if extra else {k: res[k] for k in FLUX + HR}


def assert_parity(g, o, tol=1e-9, keys=FLUX + HR, flux_floor=1e-9, hr_floor=1e-8):
    """Every element: |g - o| <= tol |o| + floor (the heating-rate floor for
    swhr / swhrc, the flux floor for every flux output)."""
    for k in keys:
        d = np.abs(g[k] - o[k])
        lim = tol * np.abs(o[k]) + (hr_floor if k in HR else flux_floor)
        bad = d > lim
        assert not bad.any(), (k, int(bad.sum()), float(np.max(d - lim)))


def mcica_oracle(c, icld, seed, irng=0, alpha=None):
    ncol, nlay = c["play"].shape
    z14 = np.zeros(14 * ncol * nlay)
    al = np.zeros(ncol * nlay) if alpha is None else np.asarray(alpha).ravel(order="F")
    m = pyoracle.mcica_subcol_sw(ncol, nlay, icld, seed, irng, *(c[k].ravel(order="F") for k in
                                                                  ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                 z14, z14 + 1.0, z14, z14, al)
    names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
    shp = {k: (112, ncol, nlay) for k in names}
    shp.update(reicmcl=(ncol, nlay), relqmcl=(ncol, nlay))
    return tuple(m[k].reshape(shp[k], order="F") for k in names)


def test_clear_sky_fp64_parity():
    c = make_columns(96, 60, 20261203)
    kw = gcm_inputs(c, icld=0, iaer=0)
    assert_parity(gpu_call(kw), oracle_call(kw))


def test_layer_counts_and_odd_ncol():
    for ncol, nlay in ((1, 40), (3, 47), (5, 72), (7, 137)):
        c = make_columns(ncol, nlay, 1000 + nlay)
        kw = gcm_inputs(c, icld=0, iaer=0)
        assert_parity(gpu_call(kw), oracle_call(kw))


def test_aerosol_iaer10_and_extra_outputs():
    c = make_columns(64, 60, 20261204, aerosol=True)
    kw = gcm_inputs(c, icld=0, iaer=10)
    g = gpu_call(kw, extra=True)
    o = oracle_call(kw, extra=True)
    assert_parity(g, o, keys=FLUX + HR + tuple(pyoracle.EXTRA_OUTPUTS))


def test_aerosol_iaer6():
    c = make_columns(32, 60, 77)
    kw = gcm_inputs(c, icld=0, iaer=6)
    kw["ecaer"] = np.random.default_rng(5).uniform(0.0, 0.3, (32, 60, 6))
    assert_parity(gpu_call(kw), oracle_call(kw))


def test_unscaled_direct_idelm0():
    c = make_columns(32, 60, 99, clouds=True)
    m = mcica_oracle(c, 2, 112)
    kw = gcm_inputs(c, icld=2, iaer=0, mcica=m)
    g = gpu_call(kw, extra=True, idelm=0)
    o = oracle_call(kw, extra=True, idelm=0)
    assert_parity(g, o, keys=FLUX + HR + ("dirdflux", "difdflux"))


@pytest.mark.parametrize("icld", [1, 2, 3, 5])
def test_mcica_subcolumns_kiss_bitexact(icld):
    c = make_columns(48, 60, 20261205, clouds=True, lat=True)
    ncol, nlay = c["play"].shape
    alpha = None
    if icld >= 4:
        alpha = pyoracle.get_alpha(ncol, nlay, icld, 1, 0.0, c["dz"].ravel(order="F"), c["lat"], 94,
                                   c["cldfrac"].ravel(order="F")).reshape((ncol, nlay), order="F")
    o = mcica_oracle(c, icld, 224, 0, alpha)
    z = np.zeros((14, ncol, nlay))
    g = gpu.mcica_subcol_sw(1, ncol, nlay, icld, 224, 0, c["play"], c["cldfrac"], c["ciwp"], c["clwp"], c["rei"],
                            c["rel"], z, z + 1.0, z, z, alpha)
    for a, b in zip(g, o):
        assert np.array_equal(a, b)
    assert 0.0 < o[0].mean() < 1.0


@pytest.mark.parametrize("icld", [2, 5])
def test_mcica_subcolumns_mt_bitexact(icld):
    c = make_columns(12, 50, 31, clouds=True, lat=True)
    ncol, nlay = c["play"].shape
    alpha = np.full((ncol, nlay), 0.7) if icld == 5 else None
    o = mcica_oracle(c, icld, 3 * 112, 1, alpha)
    z = np.zeros((14, ncol, nlay))
    g = gpu.mcica_subcol_sw(1, ncol, nlay, icld, 3 * 112, 1, c["play"], c["cldfrac"], c["ciwp"], c["clwp"],
                            c["rei"], c["rel"], z, z + 1.0, z, z, alpha)
    for a, b in zip(g, o):
        assert np.array_equal(a, b)


def test_mcica_clouds_aerosol_fp64_parity():
    # McICA clouds with aerosol at small ncol: icld=2, inflgsw=2/iceflgsw=3/liqflgsw=1, iaer=10
    c = make_columns(128, 60, 20261204, clouds=True, aerosol=True)
    m = mcica_oracle(c, 2, 112)
    kw = gcm_inputs(c, icld=2, iaer=10, mcica=m)
    assert_parity(gpu_call(kw), oracle_call(kw))


@pytest.mark.parametrize("icld", [2, 5])
def test_fused_mcica_matches_oracle(icld):
    c = make_columns(96, 60, 20261206, clouds=True, lat=True)
    ncol, nlay = c["play"].shape
    alpha = None
    if icld >= 4:
        alpha = pyoracle.get_alpha(ncol, nlay, icld, 1, 0.0, c["dz"].ravel(order="F"), c["lat"], 94,
                                   c["cldfrac"].ravel(order="F")).reshape((ncol, nlay), order="F")
    m = mcica_oracle(c, icld, 112, 0, alpha)
    kw = gcm_inputs(c, icld=icld, iaer=0, mcica=m)
    o = oracle_call(kw)
    clouds = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
                  rel=c["rel"], alpha=alpha)
    kwf = gcm_inputs(c, icld=icld, iaer=0)
    g = gpu_call(kwf, clouds=clouds)
    assert_parity(g, o)


def test_get_alpha_device():
    c = make_columns(64, 60, 8, clouds=True, lat=True)
    ncol, nlay = c["play"].shape
    for icld, idcor in ((4, 0), (5, 0), (5, 1)):
        o = pyoracle.get_alpha(ncol, nlay, icld, idcor, 2500.0, c["dz"].ravel(order="F"), c["lat"], 94,
                               c["cldfrac"].ravel(order="F")).reshape((ncol, nlay), order="F")
        g = gpu.get_alpha(1, ncol, nlay, icld, idcor, 2500.0, c["dz"], c["lat"], 94, c["cldfrac"])
        np.testing.assert_allclose(g, o, rtol=4e-16, atol=0)


def test_night_columns_clamped():
    c = make_columns(16, 60, 3, night_frac=0.5)
    kw = gcm_inputs(c, icld=0, iaer=0)
    g, o = gpu_call(kw), oracle_call(kw)
    night = kw["coszen"] <= 0
    assert night.any()
    # the reference clamps coszen to 1e-10 (rrtmg_sw_rad.f90:665-666): ~0 fluxes
    assert np.max(np.abs(g["swdflx"][night])) < 1e-6
    assert_parity(g, o)


@pytest.mark.parametrize("fused", [False, True])
def test_fp32_form_error_bounds(fused):
    # FP32 form vs the FP64 oracle: |dF| <= 0.05 W m-2, |dHR| <= 0.01 K/day
    c = make_columns(512, 60, 20261207, clouds=True, lat=True)
    ncol, nlay = c["play"].shape
    alpha = pyoracle.get_alpha(ncol, nlay, 5, 1, 0.0, c["dz"].ravel(order="F"), c["lat"], 94,
                               c["cldfrac"].ravel(order="F")).reshape((ncol, nlay), order="F")
    m = mcica_oracle(c, 5, 112, 0, alpha)
    kw = gcm_inputs(c, icld=5, iaer=0, mcica=m)
    o = oracle_call(kw)
    clouds = None
    if fused:
        clouds = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
                      rel=c["rel"], alpha=alpha)
        kw = gcm_inputs(c, icld=5, iaer=0)
    gpu.set_form(gpu.FORM_FP32)
    try:
        g = gpu_call(kw, clouds=clouds)
    finally:
        gpu.set_form(gpu.FORM_FP64)
    for k in FLUX:
        assert np.max(np.abs(g[k] - o[k])) <= 0.05, (k, float(np.max(np.abs(g[k] - o[k]))))
    for k in HR:
        assert np.max(np.abs(g[k] - o[k])) <= 0.01, (k, float(np.max(np.abs(g[k] - o[k]))))


def test_fp32_form_aerosol_error_bounds():
    c = make_columns(256, 60, 20261208, clouds=True, aerosol=True)
    m = mcica_oracle(c, 2, 112)
    kw = gcm_inputs(c, icld=2, iaer=10, mcica=m)
    o = oracle_call(kw)
    gpu.set_form(gpu.FORM_FP32)
    try:
        g = gpu_call(kw)
    finally:
        gpu.set_form(gpu.FORM_FP64)
    for k in FLUX:
        assert np.max(np.abs(g[k] - o[k])) <= 0.05, k
    for k in HR:
        assert np.max(np.abs(g[k] - o[k])) <= 0.01, k


def test_invalid_ice_size_reports_reference_error():
    c = make_columns(4, 60, 5, clouds=True)
    c["rei"] = np.full_like(c["rei"], 200.0)  # iceflgsw=3 accepts 5..140 (cldprmc:227)
    m = mcica_oracle(c, 2, 112)
    if m[1].max() == 0.0:
        pytest.skip("no ice in the sampled subcolumns")
    kw = gcm_inputs(c, icld=2, iaer=0, mcica=m)
    with pytest.raises(gpu.RRTMGError) as ei:
        gpu_call(kw)
    assert ei.value.code == 12 and "ICE GENERALIZED EFFECTIVE SIZE" in str(ei.value)


def test_empty_calls_do_nothing():
    # ncol = 0: the reference's column loop runs no iteration; every entry point returns 0
    import ctypes as C
    a = gpu.RrtmgSwArgs()
    a.ncol, a.nlay, a.icld, a.iaer = 0, 60, 2, 0
    cl = gpu.RrtmgSwClouds()
    L = gpu.lib()
    assert L.rrtmg_sw_c(C.byref(a)) == 0
    assert L.rrtmg_sw_mcica_c(C.byref(a), C.byref(cl)) == 0
    assert L.rrtmg_sw_dev_c(C.byref(a), None) == 0
    assert L.rrtmg_sw_nomcica_c(C.byref(a), C.byref(cl)) == 0
    null = C.cast(None, gpu._dp)
    assert L.mcica_subcol_sw_c(0, 60, 2, 112, 0, *([null] * 20)) == 0
    assert L.get_alpha_c(0, 60, 5, 1, C.c_double(0.0), null, null, 94, null, null) == 0
    a.ncol = -1
    assert L.rrtmg_sw_c(C.byref(a)) == 3  # RRTMG_SW_EARGS
