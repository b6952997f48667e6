"""The FP32 form's tiled kernel (layer R/T in shared memory, vertical adding
by two warps, clear and total sky, per tile of 32 subcolumns, FP64 cells
redone by a dedicated warp) against the FP64 oracle and against the scratch-based FP32 kernel.

Tolerances: |dF| <= 0.05 W m-2 and |dHR| <= 0.01 K/day against the oracle
(the FP32 form's bounds); against the scratch-based FP32 kernel, which makes
the same discrete choices, 1e-3 W m-2 and 1e-4 K/day.  The library chooses
the kernel for nlay <= 64 with idelm = 1 when its shared memory fits (every
case here asserts which kernel ran); RRTMG_SW_TILED=0 (read at
rrtmg_sw_ini_c) keeps the scratch-based kernel, and RRTMG_SW_TILE_QCAP
lowers the tiled kernel's capacity of FP64 cells per column pair so that its
fallback (pairs solved again by the scratch-based kernel) runs.
"""
import os

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
    os.environ.pop("RRTMG_SW_TILED", None)
    os.environ.pop("RRTMG_SW_TILE_QCAP", None)
    gpu.rrtmg_sw_ini(1.004e3)
    gpu.set_form(gpu.FORM_FP64)


def set_env(tiled=True, qcap=None):
    os.environ["RRTMG_SW_TILED"] = "1" if tiled else "0"
    if qcap is None:
        os.environ.pop("RRTMG_SW_TILE_QCAP", None)
    else:
        os.environ["RRTMG_SW_TILE_QCAP"] = str(qcap)
    gpu.rrtmg_sw_ini(1.004e3)


def case(ncol, nlay, seed, icld, iaer=0):
    c = make_columns(ncol, nlay, seed, clouds=icld > 0, lat=True, aerosol=iaer == 10)
    alpha = None
    if icld >= 4:
        alpha = pyoracle.get_alpha(ncol, nlay, icld, 1, 0.0, c["dz"].ravel(order="F"), c["lat"], 94,
                                   c["cldfrac"].ravel(order="F")).reshape((ncol, nlay), order="F")
    clouds = None
    if icld:
        clouds = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
                      rel=c["rel"], alpha=alpha)
    return c, clouds, alpha


def run_fp32(c, clouds, icld, iaer, bands=False, extra=False, tiled=None):
    gpu.set_form(gpu.FORM_FP32)
    try:
        res = gpu.rrtmg_sw(**gcm_inputs(c, icld=icld, iaer=iaer), clouds=clouds, extra=extra, bands=bands)
    finally:
        gpu.set_form(gpu.FORM_FP64)
    if not isinstance(res, dict):
        res = dict(zip(("swuflx", "swdflx", "swhr", "swuflxc", "swdflxc", "swhrc"), res))
    if tiled is not None:
        want = gpu.KERNEL_FP32_TILED if tiled else gpu.KERNEL_FP32
        assert gpu.last_kernel() == want, (gpu.last_kernel(), want)
    return res


def oracle(c, icld, iaer, alpha):
    ncol, nlay = c["play"].shape
    mc = None
    if icld:
        z14 = np.zeros(14 * ncol * nlay)
        al = np.zeros(ncol * nlay) if alpha is None else alpha.ravel(order="F")
        m = pyoracle.mcica_subcol_sw(ncol, nlay, icld, 112, 0, *(c[k].ravel(order="F") for k in
                                                                 ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                     z14, z14 + 1.0, z14, z14, al)
        names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
        mc = tuple(m[k] for k in names)
    kw = gcm_inputs(c, icld=icld, iaer=iaer, mcica=mc)
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS + pyoracle.MCICA_INPUTS + pyoracle.AER_INPUTS}
    out = pyoracle.rrtmg_sw(ncol, nlay, icld, iaer, inp)
    shp = {k: (ncol, nlay + 1) for k in out}
    shp.update(swhr=(ncol, nlay), swhrc=(ncol, nlay))
    return {k: v.reshape(shp[k], order="F") for k, v in out.items()}


def check_bounds(g, o, fl=0.05, hr=0.01):
    for k in FLUX:
        assert np.max(np.abs(g[k] - o[k])) <= fl, (k, float(np.max(np.abs(g[k] - o[k]))))
    for k in HR:
        assert np.max(np.abs(g[k] - o[k])) <= hr, (k, float(np.max(np.abs(g[k] - o[k]))))


@pytest.mark.parametrize("icld,iaer", [(0, 0), (2, 0), (5, 0), (2, 10)])
def test_tiled_against_oracle(icld, iaer):
    set_env(tiled=True)
    c, clouds, alpha = case(300, 60, 20261220 + icld + iaer, icld, iaer)
    g = run_fp32(c, clouds, icld, iaer, tiled=True)
    assert gpu.lib().rrtmg_sw_last_launch_count_c() == 2  # preparation + solve
    assert gpu.last_tile_slots() == 3  # 60 layers, 8 level sums: three pair slots fit
    check_bounds(g, oracle(c, icld, iaer, alpha))


@pytest.mark.parametrize("nlay", [5, 33, 47, 62])
def test_tiled_layer_counts_odd_ncol(nlay):
    set_env(tiled=True)
    c, clouds, alpha = case(37, nlay, 7000 + nlay, 2)
    check_bounds(run_fp32(c, clouds, 2, 0, tiled=True), oracle(c, 2, 0, alpha))


def test_tiled_matches_scratch_kernel_with_outputs():
    # extra (direct/diffuse, UV/NIR) and per-band outputs, tiled vs scratch-based FP32 kernel
    c, clouds, alpha = case(256, 60, 20261230, 5)
    set_env(tiled=False)
    ref = run_fp32(c, clouds, 5, 0, bands=True, extra=True, tiled=False)
    set_env(tiled=True)
    got = run_fp32(c, clouds, 5, 0, bands=True, extra=True, tiled=True)
    for k in FLUX + tuple(gpu.EXTRA_OUTPUTS) + tuple(gpu.BAND_OUTPUTS):
        assert np.max(np.abs(got[k] - ref[k])) <= 1e-3, (k, float(np.max(np.abs(got[k] - ref[k]))))
    for k in HR:
        assert np.max(np.abs(got[k] - ref[k])) <= 1e-4, (k, float(np.max(np.abs(got[k] - ref[k]))))


@pytest.mark.parametrize("extra,slots", [(False, 3), (True, 2)])
def test_tiled_is_deterministic(extra, slots):
    # three pair slots, and two when the extra outputs' 16 level sums leave no room for a third
    set_env(tiled=True)
    c, clouds, alpha = case(500, 60, 20261231, 5)
    a = run_fp32(c, clouds, 5, 0, extra=extra, tiled=True)
    assert gpu.last_tile_slots() == slots
    b = run_fp32(c, clouds, 5, 0, extra=extra, tiled=True)
    st = gpu.last_fp32_stats()
    # cloudy columns have FP64 cells; none handed back at full capacity
    assert st["redone_cells"] > 0 and st["subcolumns_swept_twice"] > 0 and st["pairs_handed_back"] == 0, st
    for k in FLUX + HR:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_tiled_overflow_fallback():
    # capacity of one FP64 cell per pair: pairs with more are solved a
    # second time by the scratch-based kernel
    c, clouds, alpha = case(400, 60, 20261232, 5)
    set_env(tiled=True, qcap=1)
    g = run_fp32(c, clouds, 5, 0, tiled=True)
    assert gpu.lib().rrtmg_sw_last_launch_count_c() == 3  # + the scratch kernel on the handed-back pairs
    st = gpu.last_fp32_stats()
    assert st["pairs_handed_back"] > 0 and st["redone_cells"] > 0, st
    check_bounds(g, oracle(c, 5, 0, alpha))
    set_env(tiled=True)


def test_tiled_shared_memory_limit():
    # 64 layers: the clear-sky kernel fits in shared memory; with McICA
    # (subcolumn masks and cloud staging) and the extra outputs (16 level sums
    # instead of 8) it does not, and the scratch kernel runs
    set_env(tiled=True)
    c, clouds, alpha = case(41, 64, 7064, 2)
    check_bounds(run_fp32(c, clouds, 2, 0, extra=True, tiled=False), oracle(c, 2, 0, alpha))
    c, clouds, alpha = case(41, 64, 7065, 0)
    check_bounds(run_fp32(c, None, 0, 0, tiled=True), oracle(c, 0, 0, None))
