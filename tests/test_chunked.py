"""Host-array calls of 32 768 columns or more on page-locked arrays run as
column chunks on two streams (transfers of one chunk overlap the solve of
another).  Columns are independent, so the outputs must equal those of one
device-pointer call on the same inputs bit for bit (tolerance 0), in both
forms, with fused KISS McICA, aerosol, the extra and per-band outputs, and
on the non-McICA path.
"""
import ctypes as C

import numpy as np
import pytest

from rrtmg_sw_gb300 import interface as gi
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

pytestmark = pytest.mark.gpu

NCOL, NLAY = 40000, 47  # chunks of 16384, 16384 and 7232 columns


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    from rrtmg_sw_gb300 import build
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    yield t
    gi.set_form(gi.FORM_FP64)


ARRAYS = ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif", "aldir", "aldif",
          "coszen")


def call(torch, kw, clouds, where, nomcica=False):
    """The request through the host entry point with pinned arrays (where =
    "pinned") or through the device entry point (where = "device")."""
    ncol, nlay = kw["ncol"], kw["nlay"]
    dev = torch.device("cuda", torch.cuda.current_device())
    keep = []

    def T(x):
        t = torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy())
        t = t.pin_memory() if where == "pinned" else t.to(dev)
        keep.append(t)
        return C.cast(C.c_void_p(t.data_ptr()), gi._dp)

    a = gi.RrtmgSwArgs()
    a.ncol, a.nlay, a.icld, a.iaer = ncol, nlay, kw["icld"], kw["iaer"]
    for k in ARRAYS:
        setattr(a, k, T(kw[k]))
    if kw["iaer"] == 10:
        for k in ("tauaer", "ssaaer", "asmaer"):
            setattr(a, k, T(kw[k]))
    a.adjes, a.dyofyr, a.scon, a.isolvar = kw["adjes"], kw["dyofyr"], kw["scon"], kw["isolvar"]
    a.inflgsw, a.iceflgsw, a.liqflgsw = kw["inflgsw"], kw["iceflgsw"], kw["liqflgsw"]
    a.idelm = 1
    shapes = {}
    for k in ("swuflx", "swdflx", "swuflxc", "swdflxc") + gi.EXTRA_OUTPUTS:
        shapes[k] = (ncol, nlay + 1)
    for k in ("swhr", "swhrc"):
        shapes[k] = (ncol, nlay)
    for k in gi.BAND_OUTPUTS:
        shapes[k] = (ncol, nlay + 1, 14)
    outs = {}
    for k, shp in shapes.items():
        t = torch.zeros(int(np.prod(shp)), dtype=torch.float64)
        t = t.pin_memory() if where == "pinned" else t.to(dev)
        outs[k] = t
        setattr(a, k, C.cast(C.c_void_p(t.data_ptr()), gi._dp))
    cl = gi.RrtmgSwClouds()
    cl.permuteseed, cl.irng = clouds.get("permuteseed", 112), 0
    for k in ("cldfrac", "ciwp", "clwp", "rei", "rel", "tauc", "ssac", "asmc", "fsfc"):
        if clouds.get(k) is not None:
            setattr(cl, k, T(clouds[k]))
    L = gi.lib()
    if where == "pinned":
        rc = (L.rrtmg_sw_nomcica_c if nomcica else L.rrtmg_sw_mcica_c)(C.byref(a), C.byref(cl))
        launches = L.rrtmg_sw_last_launch_count_c()
    else:
        s = torch.cuda.current_stream().cuda_stream
        rc = (L.rrtmg_sw_nomcica_dev_c if nomcica else L.rrtmg_sw_mcica_dev_c)(C.byref(a), C.byref(cl), C.c_void_p(s))
        launches = L.rrtmg_sw_last_launch_count_c()
    # the tiled FP32 kernel comes with its preparation kernel: two launches per solve
    launches = (launches, 2 if gi.last_kernel() == gi.KERNEL_FP32_TILED else 1)
    torch.cuda.synchronize()
    assert rc == 0
    res = {k: outs[k].cpu().numpy().reshape(shp, order="F") for k, shp in shapes.items()}
    return res, launches


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_chunked_host_call_equals_one_device_call(torch, form):
    c = make_columns(NCOL, NLAY, 20261209, clouds=True, aerosol=True)
    kw = gcm_inputs(c, icld=2, iaer=10)
    clouds = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
                  rel=c["rel"])
    gi.set_form(gi.FORM_FP64 if form == "fp64" else gi.FORM_FP32)
    try:
        h, nh = call(torch, kw, clouds, "pinned")
        d, nd = call(torch, kw, clouds, "device")
    finally:
        gi.set_form(gi.FORM_FP64)
    assert nh[0] == 3 * nh[1] and nd[0] == nd[1]  # one solve per chunk / one for the whole call
    for k in d:
        np.testing.assert_array_equal(h[k], d[k], err_msg=k)


def test_chunked_nomcica_equals_one_device_call(torch):
    # overcast layers with per-band cloud optics (inflgsw = 0), as the non-McICA driver takes them
    c = make_columns(NCOL, NLAY, 20261210, clouds=True)
    cf = (c["cldfrac"] > 0.5).astype(float)
    rng = np.random.default_rng(20261211)
    kw = gcm_inputs(c, icld=2, iaer=0)
    kw["inflgsw"] = 0
    clouds = dict(cldfrac=cf, ciwp=c["ciwp"] * cf, clwp=c["clwp"] * cf, rei=c["rei"], rel=c["rel"],
                  tauc=rng.uniform(0.0, 8.0, (14, NCOL, NLAY)) * cf[None],
                  ssac=rng.uniform(0.7, 0.999999, (14, NCOL, NLAY)), asmc=rng.uniform(0.5, 0.9, (14, NCOL, NLAY)))
    clouds["fsfc"] = clouds["asmc"] ** 2
    h, nh = call(torch, kw, clouds, "pinned", nomcica=True)
    d, _ = call(torch, kw, clouds, "device", nomcica=True)
    assert nh[0] == 3 * nh[1]
    for k in d:
        np.testing.assert_array_equal(h[k], d[k], err_msg=k)
