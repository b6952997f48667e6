"""MT19937 streams with jump-ahead (McICA irng = 1 at scale).

The reference draws one Mersenne Twister stream per call in (subcolumn,
column, layer) order (mcica_subcol_gen_sw.f90, mcica_random_numbers.f90:77-306).
The library generates it in segments that start by a jump-ahead.  Checks,
all bit-exact:
  CPU: the host jump (rrtmg_sw_mt_window_c) against the oracle's sequential
       generator at offsets across segment boundaries, and a far jump
       against a nearer jump advanced sequentially.
  GPU: the device stream for several segment sizes against the oracle's
       sequential stream; at 2^28 words, two segment sizes against each other
       and host windows at segment starts; the fused solve with irng = 1
       against the oracle's mcica_subcol_sw + rrtmg_sw (FP64 form, 1e-9
       relative element by element; FP32 form 0.05 W m-2 / 0.01 K/day), its subcolumns through
       the device mcica_subcol_sw (bit for bit) and the unfused solve of those
       (1e-12 relative).
"""
import numpy as np
import pytest

import pyoracle
from rrtmg_sw_gb300 import interface as gi
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

SCALE = 4294967295.0


def reals(words):
    return gi.mt_temper(words).astype(np.float64) / SCALE


def advance(window, k):
    """Sequential MT recurrence: the 624 raw words k steps after window."""
    e = list(int(x) for x in window)
    for i in range(k):
        u, v = e[i], e[i + 1]
        mix = (u & 0x80000000) | (v & 0x7fffffff)
        e.append(e[i + 397] ^ (mix >> 1) ^ (0x9908b0df if v & 1 else 0))
    return np.array(e[k:k + 624], dtype=np.uint32)


@pytest.mark.parametrize("seed", [112, 5489, -7])
def test_host_jump_matches_sequential_stream(seed):
    n = 1 << 21
    ref = pyoracle.mt_real(seed, n + 700)
    for off in (0, 1, 623, 624, 4095, 65536, 65536 * 3 + 11, (1 << 20) + 1, n):
        got = reals(gi.mt_window(seed, off))
        assert np.array_equal(got, ref[off:off + 624]), off


def test_far_jump_is_consistent():
    base = (1 << 40) + 12345
    w0 = gi.mt_window(224, base)
    for k in (1, 300, 1000):
        assert np.array_equal(gi.mt_window(224, base + k), advance(w0, k)), k


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    from rrtmg_sw_gb300 import build
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    pyoracle.init(1.004e3)
    yield t
    gi.set_form(gi.FORM_FP64)


def device_stream(torch, seed, n, log_seg):
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    gi.mt_stream_dev(seed, n, out.data_ptr(), log_seg, torch.cuda.current_stream().cuda_stream)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("log_seg", [10, 12, 16, 0])
def test_device_stream_matches_oracle(torch, log_seg):
    n = 3_000_017
    d = device_stream(torch, 336, n, log_seg).cpu().numpy().view(np.uint32)
    ref = pyoracle.mt_real(336, n)
    assert np.array_equal(d.astype(np.float64) / SCALE, ref)


@pytest.mark.gpu
def test_device_stream_large_segmentations_agree(torch):
    n = (1 << 28) + 4321
    a = device_stream(torch, 112, n, 0)
    b = device_stream(torch, 112, n, 20)
    assert torch.equal(a, b)
    h = a.cpu().numpy().view(np.uint32)
    del a, b
    for off in (0, 1 << 20, (1 << 24) * 3, (1 << 27) + 5, n - 624):
        assert np.array_equal(h[off:off + 624], gi.mt_temper(gi.mt_window(112, off))), off


def mcica(c, icld, seed, alpha):
    ncol, nlay = c["play"].shape
    z14 = np.zeros(14 * ncol * nlay)
    al = np.zeros(ncol * nlay) if alpha is None else alpha.ravel(order="F")
    m = pyoracle.mcica_subcol_sw(ncol, nlay, icld, seed, 1, *(c[k].ravel(order="F") for k in
                                                            ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                 z14, z14 + 1.0, z14, z14, al)
    names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
    shp = {k: (112, ncol, nlay) for k in names}
    shp.update(reicmcl=(ncol, nlay), relqmcl=(ncol, nlay))
    return tuple(m[k].reshape(shp[k], order="F") for k in names)


def oracle_solve(kw):
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS}
    for k in pyoracle.MCICA_INPUTS:
        if kw.get(k) is not None:
            inp[k] = kw[k]
    out = pyoracle.rrtmg_sw(kw["ncol"], kw["nlay"], kw["icld"], kw["iaer"], inp, adjes=kw["adjes"],
                            dyofyr=kw["dyofyr"], scon=kw["scon"], isolvar=kw["isolvar"], inflgsw=kw["inflgsw"],
                            iceflgsw=kw["iceflgsw"], liqflgsw=kw["liqflgsw"])
    ncol, nlay = kw["ncol"], kw["nlay"]
    return {k: v.reshape((ncol, nlay if k in ("swhr", "swhrc") else nlay + 1), order="F") for k, v in out.items()}


OUTS = ("swuflx", "swdflx", "swuflxc", "swdflxc", "swhr", "swhrc")


@pytest.mark.gpu
@pytest.mark.parametrize("icld", [1, 2, 3, 5])
def test_fused_mt_matches_oracle(torch, icld):
    c = make_columns(72, 60, 20261207 + icld, clouds=True, lat=True)
    ncol, nlay = c["play"].shape
    alpha = None
    if icld >= 4:
        alpha = pyoracle.get_alpha(ncol, nlay, icld, 1, 0.0, c["dz"].ravel(order="F"), c["lat"], 94,
                                   c["cldfrac"].ravel(order="F")).reshape((ncol, nlay), order="F")
    seed = 5 * 112
    m = mcica(c, icld, seed, alpha)
    o = oracle_solve(gcm_inputs(c, icld=icld, iaer=0, mcica=m))
    clouds = dict(permuteseed=seed, irng=1, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
                  rel=c["rel"], alpha=alpha)
    gi.set_form(gi.FORM_FP64)
    g = gi.rrtmg_sw(**gcm_inputs(c, icld=icld, iaer=0), clouds=clouds, extra=True)
    for k in OUTS:
        # every element within 1e-9 relative, floors 1e-9 W m-2 / 1e-8 K/day near zero
        d = np.abs(g[k] - o[k])
        bad = d > 1e-9 * np.abs(o[k]) + (1e-8 if k in ("swhr", "swhrc") else 1e-9)
        assert not bad.any(), (k, int(bad.sum()), float(np.max(d)))
    # the same subcolumns through the device McICA + the unfused solve
    z = np.zeros((14, ncol, nlay))
    md = gi.mcica_subcol_sw(1, ncol, nlay, icld, seed, 1, c["play"], c["cldfrac"], c["ciwp"], c["clwp"], c["rei"],
                            c["rel"], z, z + 1.0, z, z, alpha)
    for a, b in zip(md, m):
        assert np.array_equal(a, b)
    u = gi.rrtmg_sw(**gcm_inputs(c, icld=icld, iaer=0, mcica=md), extra=True)
    for k in OUTS:
        assert np.max(np.abs(g[k] - u[k])) <= 1e-12 * np.max(np.abs(u[k])), k
    gi.set_form(gi.FORM_FP32)
    try:
        f = gi.rrtmg_sw(**gcm_inputs(c, icld=icld, iaer=0), clouds=clouds, extra=True)
    finally:
        gi.set_form(gi.FORM_FP64)
    for k in OUTS:
        tol = 0.01 if k in ("swhr", "swhrc") else 0.05
        assert np.max(np.abs(f[k] - o[k])) <= tol, k
