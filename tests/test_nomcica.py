"""Non-McICA path: cldprop_sw + spcvrt_sw behind rrtmg_sw (rrtmg_sw_rad.nomcica.f90).

CPU: the oracle's non-McICA driver against its McICA driver with every
subcolumn set to the layer's cloud (the two reference drivers then solve the
same problem), and its partial-cloud stop.  GPU: the library against the
oracle, FP64 form to 1e-9 relative element by element, FP32 form within 0.05 W m-2 and
0.01 K/day.
"""
import numpy as np
import pytest

import pyoracle
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

FLUX = ("swuflx", "swdflx", "swuflxc", "swdflxc")
HR = ("swhr", "swhrc")


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    pyoracle.init(1.004e3)


def overcast_case(ncol, nlay, seed, inflag=2, aerosol=False):
    c = make_columns(ncol, nlay, seed, clouds=True, aerosol=aerosol)
    cf = (c["cldfrac"] > 0.5).astype(float)
    rng = np.random.default_rng(seed + 1)
    tau = rng.uniform(0.0, 8.0, (14, ncol, nlay)) * cf[None]
    ssa = rng.uniform(0.7, 0.999999, (14, ncol, nlay))
    asm = rng.uniform(0.5, 0.9, (14, ncol, nlay))
    fsf = asm ** 2
    kw = gcm_inputs(c, icld=2, iaer=10 if aerosol else 0)
    kw["inflgsw"] = inflag
    nm = dict(cldfr=cf, cicewp=c["ciwp"] * cf, cliqwp=c["clwp"] * cf, reice=c["rei"], reliq=c["rel"],
              taucld=tau, ssacld=ssa, asmcld=asm, fsfcld=fsf)
    return c, kw, nm


def oracle_nomcica(kw, nm):
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS}
    for k in pyoracle.AER_INPUTS:
        if kw.get(k) is not None:
            inp[k] = kw[k]
    for k, v in nm.items():
        inp[k] = np.asfortranarray(v).ravel(order="F")
    out = pyoracle.rrtmg_sw(kw["ncol"], kw["nlay"], kw["icld"], kw["iaer"], inp, inflgsw=kw["inflgsw"],
                            iceflgsw=kw["iceflgsw"], liqflgsw=kw["liqflgsw"], nomcica=True)
    ncol, nlay = kw["ncol"], kw["nlay"]
    shp = {k: (ncol, nlay + 1) for k in FLUX}
    shp.update({k: (ncol, nlay) for k in HR})
    return {k: out[k].reshape(shp[k], order="F") for k in FLUX + HR}


def oracle_mcica_equivalent(kw, nm):
    """The McICA driver with every subcolumn equal to the layer's cloud."""
    ncol, nlay = kw["ncol"], kw["nlay"]
    ngb = np.repeat(np.arange(14), [6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12])
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS}
    g = lambda x: np.broadcast_to(x[None], (112, ncol, nlay))
    inp["cldfmcl"] = g(nm["cldfr"])
    inp["ciwpmcl"] = g(nm["cicewp"])
    inp["clwpmcl"] = g(nm["cliqwp"])
    inp["taucmcl"] = nm["taucld"][ngb]
    inp["ssacmcl"] = nm["ssacld"][ngb]
    inp["asmcmcl"] = nm["asmcld"][ngb]
    inp["fsfcmcl"] = nm["fsfcld"][ngb]
    inp["reicmcl"], inp["relqmcl"] = nm["reice"], nm["reliq"]
    inp = {k: np.asfortranarray(v).ravel(order="F") for k, v in inp.items()}
    out = pyoracle.rrtmg_sw(ncol, nlay, kw["icld"], kw["iaer"], inp, inflgsw=kw["inflgsw"],
                            iceflgsw=kw["iceflgsw"], liqflgsw=kw["liqflgsw"])
    shp = {k: (ncol, nlay + 1) for k in FLUX}
    shp.update({k: (ncol, nlay) for k in HR})
    return {k: out[k].reshape(shp[k], order="F") for k in FLUX + HR}


@pytest.mark.parametrize("inflag", [0, 2])
def test_oracle_nomcica_equals_overcast_mcica(inflag):
    _, kw, nm = overcast_case(12, 40, 31, inflag=inflag)
    a, b = oracle_nomcica(kw, nm), oracle_mcica_equivalent(kw, nm)
    for k in FLUX + HR:
        np.testing.assert_allclose(a[k], b[k], rtol=1e-12, atol=1e-12, err_msg=k)


def test_oracle_nomcica_partial_cloud_stops():
    _, kw, nm = overcast_case(4, 30, 32)
    nm["cldfr"] = nm["cldfr"].copy()
    nm["cldfr"][1, 10] = 0.5
    with pytest.raises(RuntimeError, match="32"):
        oracle_nomcica(kw, nm)


def gpu_nomcica(kw, nm, form):
    from rrtmg_sw_gb300 import interface as gpu
    gpu.set_form(form)
    clouds = dict(cldfrac=nm["cldfr"], ciwp=nm["cicewp"], clwp=nm["cliqwp"], rei=nm["reice"], rel=nm["reliq"],
                  tauc=nm["taucld"], ssac=nm["ssacld"], asmc=nm["asmcld"], fsfc=nm["fsfcld"])
    res = gpu.rrtmg_sw(**kw, extra=True, clouds=clouds, nomcica=True)
    return {k: res[k] for k in FLUX + HR}


@pytest.fixture(scope="module")
def gpu_lib():
    from rrtmg_sw_gb300 import build, interface as gpu
    build.build()
    gpu.rrtmg_sw_ini(1.004e3)
    yield gpu
    gpu.set_form(gpu.FORM_FP64)


@pytest.mark.gpu
@pytest.mark.parametrize("inflag,aerosol", [(2, False), (0, False), (2, True)])
def test_gpu_nomcica_fp64_parity(gpu_lib, inflag, aerosol):
    _, kw, nm = overcast_case(67, 60, 33 + inflag, inflag=inflag, aerosol=aerosol)
    g, o = gpu_nomcica(kw, nm, gpu_lib.FORM_FP64), oracle_nomcica(kw, nm)
    for k in FLUX + HR:
        # every element within 1e-9 relative, floors 1e-9 W m-2 / 1e-8 K/day near zero
        d = np.abs(g[k] - o[k])
        bad = d > 1e-9 * np.abs(o[k]) + (1e-8 if k in HR else 1e-9)
        assert not bad.any(), (k, int(bad.sum()), float(np.max(d)))


@pytest.mark.gpu
def test_gpu_nomcica_fp32_bounds(gpu_lib):
    _, kw, nm = overcast_case(256, 60, 35)
    g, o = gpu_nomcica(kw, nm, gpu_lib.FORM_FP32), oracle_nomcica(kw, nm)
    for k in FLUX:
        assert np.max(np.abs(g[k] - o[k])) <= 0.05, k
    for k in HR:
        assert np.max(np.abs(g[k] - o[k])) <= 0.01, k


@pytest.mark.gpu
def test_gpu_nomcica_partial_cloud_error(gpu_lib):
    _, kw, nm = overcast_case(8, 30, 36)
    nm["cldfr"] = nm["cldfr"].copy()
    nm["cldfr"][3, 12] = 0.4
    with pytest.raises(gpu_lib.RRTMGError) as e:
        gpu_nomcica(kw, nm, gpu_lib.FORM_FP64)
    assert e.value.code == 32
