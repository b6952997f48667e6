"""Batched solve: many instances with different ncol and nlay in one
persistent launch, sunlit columns compacted on the device, replayed from a
CUDA graph (rrtmg_sw_batch_plan_c / rrtmg_sw_batch_run_c).

Every instance is compared with the single-instance device entry point
(rrtmg_sw_mcica_dev_c) on the same inputs.  The batch kernel runs the same
per-column code, over tiles of 2 or 4 columns per CTA (the autotuner's
choice; the per-column arithmetic and the order of the g-point sums do not
depend on the tile).  Each tile is also checked on its own.  The FP64 form is compiled without FMA contraction, so
its sunlit columns must agree bit for bit (tolerance 0); the FP32 form lets
the compiler contract each kernel's inlined copy of that code its own way, so
its sunlit columns must agree to 1e-6 relative (a few FP32 roundings).
Night columns are zero in the batch and within 1e-6 of zero in the single
call (the reference clamps mu0 to 1e-10).
"""
import ctypes as C
import os

import numpy as np
import pytest

from rrtmg_sw_gb300 import interface as gi
from rrtmg_sw_gb300.synthetic import make_columns

pytestmark = pytest.mark.gpu

OUTS = ("swuflx", "swdflx", "swuflxc", "swdflxc", "swhr", "swhrc")
IN_ARGS = ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif", "aldir",
           "aldif", "coszen")
SHAPES = ((37, 40), (512, 47), (1000, 60), (64, 72), (200, 91), (3, 137))


@pytest.fixture(scope="module")
def torch():
    # the batch launch runs the scratch-based kernels, so the single calls it
    # is compared with bit for bit use them too (RRTMG_SW_TILED=0)
    t = pytest.importorskip("torch")
    from rrtmg_sw_gb300 import build
    build.build()
    os.environ["RRTMG_SW_TILED"] = "0"
    gi.rrtmg_sw_ini(1.004e3)
    yield t
    os.environ.pop("RRTMG_SW_TILED", None)
    gi.rrtmg_sw_ini(1.004e3)
    gi.set_form(gi.FORM_FP64)


class Instance:
    """Device copies of one seeded instance with McICA clouds and night columns."""

    def __init__(self, torch, ncol, nlay, seed, bad_rei=False):
        c = make_columns(ncol, nlay, seed, clouds=True, night_frac=0.4)
        if bad_rei:
            c["rei"] = np.full_like(c["rei"], 400.0)
        self.sun = c["coszen"] > 0.0
        dev = torch.device("cuda", torch.cuda.current_device())
        T = lambda x: torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).to(dev)
        self.t = {k: T(c[k]) for k in IN_ARGS + ("cldfrac", "ciwp", "clwp", "rei", "rel")}
        for k in OUTS:
            nl = nlay if k in ("swhr", "swhrc") else nlay + 1
            self.t[k] = torch.empty(ncol * nl, dtype=torch.float64, device=dev)
        ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), gi._dp)
        a = gi.RrtmgSwArgs()
        a.ncol, a.nlay, a.icld, a.iaer = ncol, nlay, 2, 0
        for k in IN_ARGS + OUTS:
            setattr(a, k, ptr(self.t[k]))
        a.adjes, a.dyofyr, a.scon, a.isolvar = 1.0, 0, 1360.85, 0
        a.inflgsw, a.iceflgsw, a.liqflgsw = 2, 3, 1
        a.idelm = 1
        cl = gi.RrtmgSwClouds()
        cl.permuteseed, cl.irng = 112, 0
        for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
            setattr(cl, k, ptr(self.t[k]))
        self.args, self.clouds, self.ncol, self.nlay = a, cl, ncol, nlay

    def fill_nan(self):
        for k in OUTS:
            self.t[k].fill_(float("nan"))

    def outputs(self):
        res = {}
        for k in OUTS:
            nl = self.nlay if k in ("swhr", "swhrc") else self.nlay + 1
            res[k] = self.t[k].cpu().numpy().reshape((self.ncol, nl), order="F")
        return res


def single(torch, inst):
    inst.fill_nan()
    s = torch.cuda.current_stream().cuda_stream
    rc = gi.lib().rrtmg_sw_mcica_dev_c(C.byref(inst.args), C.byref(inst.clouds), C.c_void_p(s))
    torch.cuda.synchronize()
    assert rc == 0
    return inst.outputs()


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_batch_matches_single_instance_calls(torch, form):
    gi.set_form(gi.FORM_FP64 if form == "fp64" else gi.FORM_FP32)
    insts = [Instance(torch, nc, nl, 900 + i) for i, (nc, nl) in enumerate(SHAPES)]
    ref = [single(torch, x) for x in insts]
    s = torch.cuda.current_stream().cuda_stream
    plan = gi.BatchPlan([x.args for x in insts], [x.clouds for x in insts], stream=s)
    info = plan.info()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert info["grid"] % sms == 0 and len(info["trial_ms"]) >= 2
    # the autotuner timed both tiles (2 and 4 columns x 112 g-points per CTA:
    # both fit the 137-layer instance's shared memory) and kept a timed one
    assert len(info["trials"]) == len(info["trial_ms"])
    assert {t[0] for t in info["trials"]} == {2, 4}, info["trials"]
    assert info["tile"][1] == 112 and (info["tile"][0], info["deepest_first"], info["grid"] // sms) in info["trials"]
    for run in range(2):  # graph replays
        for x in insts:
            x.fill_nan()
        plan.run(s)
        torch.cuda.synchronize()
        for x, r in zip(insts, ref):
            got = x.outputs()
            for k in OUTS:
                if form == "fp64":
                    np.testing.assert_array_equal(got[k][x.sun], r[k][x.sun], err_msg="run %d %s" % (run, k))
                else:
                    np.testing.assert_allclose(got[k][x.sun], r[k][x.sun], rtol=1e-6, atol=1e-9,
                                               err_msg="run %d %s" % (run, k))
                assert np.all(got[k][~x.sun] == 0.0), (run, k)
                assert np.all(np.abs(r[k][~x.sun]) <= 1e-6), (run, k)
    plan.close()


@pytest.mark.parametrize("tile", [2, 4])
def test_batch_each_tile_matches_single_calls(torch, tile):
    # RRTMG_SW_BATCH_TILE (read at rrtmg_sw_ini_c) keeps one tile: both give
    # the single calls' FP64 values bit for bit
    gi.set_form(gi.FORM_FP64)
    insts = [Instance(torch, nc, nl, 960 + i) for i, (nc, nl) in enumerate(SHAPES)]
    ref = [single(torch, x) for x in insts]
    os.environ["RRTMG_SW_BATCH_TILE"] = str(tile)
    try:
        gi.rrtmg_sw_ini(1.004e3)
        s = torch.cuda.current_stream().cuda_stream
        plan = gi.BatchPlan([x.args for x in insts], [x.clouds for x in insts], stream=s)
    finally:
        os.environ.pop("RRTMG_SW_BATCH_TILE", None)
        gi.rrtmg_sw_ini(1.004e3)
    info = plan.info()
    assert info["tile"] == (tile, 112) and {t[0] for t in info["trials"]} == {tile}, info
    for x in insts:
        x.fill_nan()
    plan.run(s)
    torch.cuda.synchronize()
    for x, r in zip(insts, ref):
        got = x.outputs()
        for k in OUTS:
            np.testing.assert_array_equal(got[k][x.sun], r[k][x.sun], err_msg="tile %d %s" % (tile, k))
            assert np.all(got[k][~x.sun] == 0.0), k
    plan.close()


def test_batch_reports_instance_errors(torch):
    gi.set_form(gi.FORM_FP64)
    insts = [Instance(torch, 64, 60, 950), Instance(torch, 32, 47, 951, bad_rei=True)]
    s = torch.cuda.current_stream().cuda_stream
    # planning runs the autotuner's trials, which already meet the bad instance
    with pytest.raises(gi.RRTMGError) as e:
        plan = gi.BatchPlan([x.args for x in insts], [x.clouds for x in insts], stream=s)
        plan.run(s)
    assert e.value.code == 12
