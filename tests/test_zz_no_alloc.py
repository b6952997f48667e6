"""rrtmg_sw_static_dev_c, the allocation-free device solve, against the
allocating device entry points (rrtmg_sw_mcica_dev_c, rrtmg_sw_dev_c),
called through the C ABI on device pointers.

Both entry points run the same kernel; only the number of resident CTAs and
the scratch address differ, and every column pair is solved by one CTA in the
same order of operations.  Tolerance: 0 -- results must be bit-identical.
This file is collected last so that it also runs after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

from rrtmg_sw_gb300 import interface as gi
from rrtmg_sw_gb300.synthetic import make_columns

pytestmark = pytest.mark.gpu

OUTS = ("swuflx", "swdflx", "swuflxc", "swdflxc", "swhr", "swhrc")
IN_ARGS = ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif", "aldir",
           "aldif", "coszen")


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    from rrtmg_sw_gb300 import build
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    yield t
    gi.set_form(gi.FORM_FP64)


class DevCase:
    """Device copies of one seeded case plus argument structs pointing at them.
    ``more`` also requests the eight extra outputs and the per-band fluxes."""

    def __init__(self, torch, ncol, nlay, seed, icld, more=False, irng=0):
        c = make_columns(ncol, nlay, seed, clouds=icld > 0)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.t = {}
        self.outs = OUTS + (gi.EXTRA_OUTPUTS + gi.BAND_OUTPUTS if more else ())

        def T(x):
            return torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).to(dev)

        for k in IN_ARGS:
            self.t[k] = T(c[k])
        for k in self.outs:
            n = ncol * (nlay if k in ("swhr", "swhrc") else nlay + 1)
            if k in gi.BAND_OUTPUTS:
                n *= 14
            self.t[k] = torch.empty(n, dtype=torch.float64, device=dev)
        ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), gi._dp)
        a = gi.RrtmgSwArgs()
        a.ncol, a.nlay, a.icld, a.iaer = ncol, nlay, icld, 0
        for k in IN_ARGS + self.outs:
            setattr(a, k, ptr(self.t[k]))
        a.adjes, a.dyofyr, a.scon, a.isolvar = 1.0, 0, 1360.85, 0
        a.inflgsw, a.iceflgsw, a.liqflgsw = 2, 3, 1
        a.idelm = 1
        self.args = a
        self.clouds = None
        if icld > 0:
            for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
                self.t[k] = T(c[k])
            cl = gi.RrtmgSwClouds()
            cl.permuteseed, cl.irng = 112, irng
            for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
                setattr(cl, k, ptr(self.t[k]))
            self.clouds = cl
        self.stream = torch.cuda.current_stream(dev).cuda_stream
        self.torch = torch

    def run(self, entry):
        """Fill the outputs with NaN, call ``entry`` through the C ABI, return
        (status, host copies of the outputs)."""
        for k in self.outs:
            self.t[k].fill_(float("nan"))
        L = gi.lib()
        cp = C.byref(self.clouds) if self.clouds is not None else None
        if entry == "static":
            rc = L.rrtmg_sw_static_dev_c(C.byref(self.args), cp, C.c_void_p(self.stream))
        elif cp is not None:
            rc = L.rrtmg_sw_mcica_dev_c(C.byref(self.args), cp, C.c_void_p(self.stream))
        else:
            rc = L.rrtmg_sw_dev_c(C.byref(self.args), C.c_void_p(self.stream))
        self.torch.cuda.synchronize()
        return rc, {k: self.t[k].cpu().numpy() for k in self.outs}


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_static_matches_allocating_entry_fused_mcica(torch, form):
    # 1000 columns = 500 column pairs: more pairs than the scratch slots that
    # fit for the FP64 form at 60 layers, so the persistent loop is exercised.
    gi.set_form(gi.FORM_FP64 if form == "fp64" else gi.FORM_FP32)
    case = DevCase(torch, 1000, 60, 20261211, icld=2)
    rc, ref = case.run("alloc")
    assert rc == 0, gi.lib().rrtmg_sw_errstr_c(rc)
    for call in range(2):
        free_before = torch.cuda.mem_get_info()[0]
        rc, got = case.run("static")
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0, (call, gi.lib().rrtmg_sw_errstr_c(rc))
        for k in OUTS:
            assert np.all(np.isfinite(got[k])), (call, k)
            np.testing.assert_array_equal(got[k], ref[k], err_msg="call %d %s" % (call, k))
        if call == 1:
            # the second call finds the area already set up: no device memory taken
            assert free_after >= free_before - (2 << 20), (free_before, free_after)


def test_static_matches_allocating_entry_clear_sky(torch):
    gi.set_form(gi.FORM_FP64)
    case = DevCase(torch, 257, 47, 20261212, icld=0)
    rc, ref = case.run("alloc")
    assert rc == 0
    for call in range(2):
        rc, got = case.run("static")
        assert rc == 0, call
        for k in OUTS:
            np.testing.assert_array_equal(got[k], ref[k], err_msg="call %d %s" % (call, k))


def test_static_rejects_request_beyond_scratch(torch):
    # FP64, idelm=1, 200 layers: 200*14*224*8 B = 5.0 MB per slot; 400 columns
    # (200 pairs) need one slot per SM, and fewer than 152 fit in 256 MiB ->
    # RRTMG_SW_ESCRATCH and nothing runs.
    gi.set_form(gi.FORM_FP64)
    case = DevCase(torch, 400, 200, 20261213, icld=0)
    rc, got = case.run("static")
    assert rc == 5
    assert "STATIC SCRATCH" in gi.lib().rrtmg_sw_errstr_c(rc).decode()
    for k in OUTS:
        assert np.all(np.isnan(got[k])), k


def test_static_small_deep_call_fits(torch):
    # 4 columns x 200 layers: 2 column pairs need 2 of the 51 slots that fit,
    # so the call runs and gives the allocating entry's results bit for bit.
    gi.set_form(gi.FORM_FP64)
    case = DevCase(torch, 4, 200, 20261213, icld=0)
    rc, ref = case.run("alloc")
    assert rc == 0
    rc, got = case.run("static")
    assert rc == 0, gi.lib().rrtmg_sw_errstr_c(rc)
    for k in OUTS:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


def test_static_rejects_mt19937(torch):
    # irng = 1 needs a device buffer for the call's MT stream: RRTMG_SW_EIRNG,
    # and the outputs are left untouched
    gi.set_form(gi.FORM_FP64)
    case = DevCase(torch, 8, 60, 20261214, icld=2, irng=1)
    rc, got = case.run("static")
    assert rc == 31
    for k in OUTS:
        assert np.all(np.isnan(got[k])), k


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_static_extra_and_band_outputs(torch, form):
    # the eight direct/diffuse/UV/NIR outputs and the per-band fluxes through
    # the static entry, bit for bit against rrtmg_sw_mcica_dev_c
    gi.set_form(gi.FORM_FP64 if form == "fp64" else gi.FORM_FP32)
    case = DevCase(torch, 66, 60, 20261215, icld=2, more=True)
    rc, ref = case.run("alloc")
    assert rc == 0
    rc, got = case.run("static")
    assert rc == 0
    for k in case.outs:
        assert np.all(np.isfinite(got[k])), k
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
