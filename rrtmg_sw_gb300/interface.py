"""Python mirror of RRTMG_SW's GCM interface on top of the C ABI.

Same routine names, argument names and meanings as the reference:

* ``rrtmg_sw_ini(cpdair)``                     -- rrtmg_sw_init.f90:47
* ``rrtmg_sw(ncol, nlay, icld, iaer, play, ...)`` -- rrtmg_sw_rad.f90:99-111
* ``mcica_subcol_sw(iplon, ncol, nlay, ...)``  -- mcica_subcol_gen_sw.f90:181-185
* ``get_alpha(iplon, ncol, nlayers, ...)``     -- mcica_subcol_gen_sw.f90:66-67

Arrays are NumPy arrays with the reference's Fortran shapes, e.g. ``play``
is ``(ncol, nlay)``, ``cldfmcl`` is ``(ngptsw, ncol, nlay)``; they are passed
in column-major order.  Outputs are returned as Fortran-ordered arrays.
Errors the reference reports with ``stop`` raise :class:`RRTMGError` with the
same message.  Every call runs on the GPU through ``librrtmg_sw_gb300.so``;
there is no CPU path.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "librrtmg_sw_gb300.so")
NGPTSW = 112
NBNDSW = 14

FORM_FP64 = 0
FORM_FP32 = 1

_dp = C.POINTER(C.c_double)


class RRTMGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rrtmg_sw error %d: %s" % (code, msg))
        self.code = code


class RrtmgSwArgs(C.Structure):
    """``rrtmg_sw_args`` of include/rrtmg_sw_gb300.h."""
    _fields_ = [
        ("ncol", C.c_int32), ("nlay", C.c_int32), ("icld", C.c_int32), ("iaer", C.c_int32),
        ("play", _dp), ("plev", _dp), ("tlay", _dp), ("tlev", _dp), ("tsfc", _dp),
        ("h2ovmr", _dp), ("o3vmr", _dp), ("co2vmr", _dp), ("ch4vmr", _dp), ("n2ovmr", _dp), ("o2vmr", _dp),
        ("asdir", _dp), ("asdif", _dp), ("aldir", _dp), ("aldif", _dp),
        ("coszen", _dp), ("adjes", C.c_double), ("dyofyr", C.c_int32), ("scon", C.c_double),
        ("isolvar", C.c_int32), ("inflgsw", C.c_int32), ("iceflgsw", C.c_int32), ("liqflgsw", C.c_int32),
        ("cldfmcl", _dp), ("taucmcl", _dp), ("ssacmcl", _dp), ("asmcmcl", _dp), ("fsfcmcl", _dp),
        ("ciwpmcl", _dp), ("clwpmcl", _dp), ("reicmcl", _dp), ("relqmcl", _dp),
        ("tauaer", _dp), ("ssaaer", _dp), ("asmaer", _dp), ("ecaer", _dp),
        ("swuflx", _dp), ("swdflx", _dp), ("swhr", _dp), ("swuflxc", _dp), ("swdflxc", _dp), ("swhrc", _dp),
        ("bndsolvar", _dp), ("indsolvar", _dp), ("solcycfrac", _dp),
        ("dirdflux", _dp), ("difdflux", _dp), ("uvdflx", _dp), ("nidflx", _dp),
        ("dirdnuv", _dp), ("difdnuv", _dp), ("dirdnir", _dp), ("difdnir", _dp),
        ("idelm", C.c_int32), ("nthreads", C.c_int32),
        ("bndfu", _dp), ("bndfd", _dp), ("bndfddir", _dp), ("bndcu", _dp), ("bndcd", _dp),
    ]


class RrtmgSwAdArgs(C.Structure):
    """``rrtmg_sw_ad_args`` of include/rrtmg_sw_gb300.h."""
    _fields_ = [
        ("w_toa_up", C.c_double), ("w_sfc_net", C.c_double), ("w_hr_sum", C.c_double),
        ("store", C.c_int32), ("pad", C.c_int32), ("J", _dp), ("dJ", _dp),
        ("tlay", _dp), ("h2ovmr", _dp), ("o3vmr", _dp), ("clwp", _dp), ("ciwp", _dp),
        ("asdir", _dp), ("asdif", _dp), ("aldir", _dp), ("aldif", _dp),
    ]


class RrtmgSwClouds(C.Structure):
    """``rrtmg_sw_clouds`` of include/rrtmg_sw_gb300.h."""
    _fields_ = [
        ("permuteseed", C.c_int32), ("irng", C.c_int32),
        ("cldfrac", _dp), ("ciwp", _dp), ("clwp", _dp), ("rei", _dp), ("rel", _dp),
        ("tauc", _dp), ("ssac", _dp), ("asmc", _dp), ("fsfc", _dp), ("alpha", _dp),
    ]


EXTRA_OUTPUTS = ("dirdflux", "difdflux", "uvdflx", "nidflx", "dirdnuv", "difdnuv", "dirdnir", "difdnir")
BAND_OUTPUTS = ("bndfu", "bndfd", "bndfddir", "bndcu", "bndcd")
_lib = None


def lib():
    """Load the CUDA library; raise if it has not been built."""
    global _lib
    if _lib is None:
        # RRTMG_SW_LIB selects another build of the library (e.g. the
        # bounds-check build, rrtmg_sw_gb300.build.build(bounds_check=True))
        path = os.environ.get("RRTMG_SW_LIB", LIB_PATH)
        if not os.path.exists(path):
            raise RuntimeError("%s is not built (run rrtmg_sw_gb300.build.build())" % path)
        L = C.CDLL(path)
        L.rrtmg_sw_ini_c.argtypes = [C.c_double]
        L.rrtmg_sw_c.argtypes = [C.POINTER(RrtmgSwArgs)]
        L.rrtmg_sw_dev_c.argtypes = [C.POINTER(RrtmgSwArgs), C.c_void_p]
        L.rrtmg_sw_mcica_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds)]
        L.rrtmg_sw_mcica_dev_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds), C.c_void_p]
        L.rrtmg_sw_nomcica_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds)]
        L.rrtmg_sw_ad_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds), C.POINTER(RrtmgSwAdArgs)]
        L.rrtmg_sw_tl_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds), C.POINTER(RrtmgSwAdArgs)]
        L.rrtmg_sw_batch_plan_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds), C.c_int32, C.c_void_p,
                                            C.POINTER(C.c_void_p)]
        L.rrtmg_sw_batch_run_c.argtypes = [C.c_void_p, C.c_void_p]
        L.rrtmg_sw_batch_info_c.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.rrtmg_sw_batch_tile_c.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.rrtmg_sw_batch_free_c.argtypes = [C.c_void_p]
        L.rrtmg_sw_nomcica_dev_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds), C.c_void_p]
        L.rrtmg_sw_static_dev_c.argtypes = [C.POINTER(RrtmgSwArgs), C.POINTER(RrtmgSwClouds), C.c_void_p]
        L.mcica_subcol_sw_c.argtypes = [C.c_int32] * 5 + [_dp] * 11 + [_dp] * 9
        L.get_alpha_c.argtypes = [C.c_int32] * 4 + [C.c_double, _dp, _dp, C.c_int32, _dp, _dp]
        L.rrtmg_sw_set_form_c.argtypes = [C.c_int32]
        L.rrtmg_sw_setcoef_c.argtypes = [C.POINTER(RrtmgSwArgs)] + [C.POINTER(C.c_int32)] * 6
        L.rrtmg_sw_mt_window_c.argtypes = [C.c_int32, C.c_uint64, C.POINTER(C.c_uint32)]
        L.rrtmg_sw_mt_stream_dev_c.argtypes = [C.c_int32, C.c_uint64, C.c_void_p, C.c_int32, C.c_void_p]
        L.rrtmg_sw_errstr_c.restype = C.c_char_p
        L.rrtmg_sw_errstr_c.argtypes = [C.c_int32]
        L.rrtmg_sw_last_cuda_error_c.restype = C.c_char_p
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        msg = lib().rrtmg_sw_errstr_c(rc).decode()
        if rc == 4:
            msg += " (" + lib().rrtmg_sw_last_cuda_error_c().decode() + ")"
        raise RRTMGError(rc, msg)


def _f(a, shape=None):
    """Fortran-ordered FP64 copy (or view) of an input array."""
    if a is None:
        return None
    x = np.asfortranarray(np.asarray(a, dtype=np.float64))
    if shape is not None and x.shape != tuple(shape):
        x = np.asfortranarray(x.reshape(shape, order="F"))
    return x


def _p(x):
    return None if x is None else x.ctypes.data_as(_dp)


def rrtmg_sw_ini(cpdair=1.004e3):
    """Load the coefficient tables onto the current GPU (rrtmg_sw_ini)."""
    _check(lib().rrtmg_sw_ini_c(C.c_double(cpdair)))


def set_form(form):
    """Select the arithmetic form: FORM_FP64 (default) or FORM_FP32."""
    _check(lib().rrtmg_sw_set_form_c(int(form)))


def rrtmg_sw(ncol, nlay, icld, iaer, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr,
             o2vmr, asdir, asdif, aldir, aldif, coszen, adjes, dyofyr, scon, isolvar, inflgsw, iceflgsw,
             liqflgsw, cldfmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl,
             tauaer, ssaaer, asmaer, ecaer, bndsolvar=None, indsolvar=None, solcycfrac=None, idelm=1,
             extra=False, clouds=None, nomcica=False, bands=False):
    """rrtmg_sw (rrtmg_sw_rad.f90:99-111).

    Returns ``(swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc)`` with shapes
    (ncol, nlay+1) and (ncol, nlay), or, with ``extra=True``, a dict that
    also holds the direct/diffuse and UV/near-IR fluxes; ``bands=True`` adds
    the per-band fluxes BAND_OUTPUTS, shape (ncol, nlay+1, 14).  ``clouds`` (a dict
    of mcica_subcol_sw's physical inputs plus ``permuteseed``) selects the
    fused path, in which the subcolumn arrays may be None.  With
    ``nomcica=True``, ``clouds`` holds the cloud arguments of the non-McICA
    rrtmg_sw (rrtmg_sw_rad.nomcica.f90:97-109) -- cldfrac (cldfr), ciwp
    (cicewp), clwp (cliqwp), rei (reice), rel (reliq), tauc/ssac/asmc/fsfc
    (taucld .. fsfcld) -- and the solve is cldprop_sw + spcvrt_sw.
    """
    cl, cl1 = (ncol, nlay), (ncol, nlay + 1)
    gcl = (NGPTSW, ncol, nlay)
    keep = {}
    a = RrtmgSwArgs()
    a.ncol, a.nlay, a.icld, a.iaer = ncol, nlay, icld, iaer
    for name, val, shp in (("play", play, cl), ("plev", plev, cl1), ("tlay", tlay, cl), ("tlev", tlev, cl1),
                           ("tsfc", tsfc, (ncol,)), ("h2ovmr", h2ovmr, cl), ("o3vmr", o3vmr, cl),
                           ("co2vmr", co2vmr, cl), ("ch4vmr", ch4vmr, cl), ("n2ovmr", n2ovmr, cl),
                           ("o2vmr", o2vmr, cl), ("asdir", asdir, (ncol,)), ("asdif", asdif, (ncol,)),
                           ("aldir", aldir, (ncol,)), ("aldif", aldif, (ncol,)), ("coszen", coszen, (ncol,)),
                           ("cldfmcl", cldfmcl, gcl), ("taucmcl", taucmcl, gcl), ("ssacmcl", ssacmcl, gcl),
                           ("asmcmcl", asmcmcl, gcl), ("fsfcmcl", fsfcmcl, gcl), ("ciwpmcl", ciwpmcl, gcl),
                           ("clwpmcl", clwpmcl, gcl), ("reicmcl", reicmcl, cl), ("relqmcl", relqmcl, cl),
                           ("tauaer", tauaer, (ncol, nlay, NBNDSW)), ("ssaaer", ssaaer, (ncol, nlay, NBNDSW)),
                           ("asmaer", asmaer, (ncol, nlay, NBNDSW)), ("ecaer", ecaer, (ncol, nlay, 6))):
        keep[name] = _f(val, shp)
        setattr(a, name, _p(keep[name]))
    a.adjes, a.dyofyr, a.scon, a.isolvar = adjes, dyofyr, scon, isolvar
    a.inflgsw, a.iceflgsw, a.liqflgsw = inflgsw, iceflgsw, liqflgsw
    if bndsolvar is not None:
        keep["bndsolvar"] = _f(bndsolvar)
        a.bndsolvar = _p(keep["bndsolvar"])
    if indsolvar is not None:
        keep["indsolvar"] = _f(indsolvar)
        a.indsolvar = _p(keep["indsolvar"])
    if solcycfrac is not None:
        keep["solcycfrac"] = _f([solcycfrac])
        a.solcycfrac = _p(keep["solcycfrac"])
    out = {k: np.zeros(cl1, order="F") for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    out.update({k: np.zeros(cl, order="F") for k in ("swhr", "swhrc")})
    if extra:
        out.update({k: np.zeros(cl1, order="F") for k in EXTRA_OUTPUTS})
    if bands:
        out.update({k: np.zeros((ncol, nlay + 1, NBNDSW), order="F") for k in BAND_OUTPUTS})
    for k, v in out.items():
        setattr(a, k, _p(v))
    a.idelm = idelm
    if clouds is None:
        _check(lib().rrtmg_sw_c(C.byref(a)))
    else:
        c = RrtmgSwClouds()
        c.permuteseed = clouds.get("permuteseed", NGPTSW)
        c.irng = clouds.get("irng", 0)
        for name, shp in (("cldfrac", cl), ("ciwp", cl), ("clwp", cl), ("rei", cl), ("rel", cl),
                          ("tauc", (NBNDSW, ncol, nlay)), ("ssac", (NBNDSW, ncol, nlay)),
                          ("asmc", (NBNDSW, ncol, nlay)), ("fsfc", (NBNDSW, ncol, nlay)), ("alpha", cl)):
            keep["c_" + name] = _f(clouds.get(name), shp)
            setattr(c, name, _p(keep["c_" + name]))
        if nomcica:
            _check(lib().rrtmg_sw_nomcica_c(C.byref(a), C.byref(c)))
        else:
            _check(lib().rrtmg_sw_mcica_c(C.byref(a), C.byref(c)))
    if extra or bands:
        return out
    return tuple(out[k] for k in ("swuflx", "swdflx", "swhr", "swuflxc", "swdflxc", "swhrc"))


def mcica_subcol_sw(iplon, ncol, nlay, icld, permuteseed, irng, play, cldfrac, ciwp, clwp, rei, rel, tauc,
                    ssac, asmc, fsfc, alpha=None):
    """mcica_subcol_sw (mcica_subcol_gen_sw.f90:181-296).

    Returns ``(cldfmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, taucmcl, ssacmcl,
    asmcmcl, fsfcmcl)``; ``irng`` 0 = KISS, 1 = Mersenne Twister.
    """
    cl, bcl, gcl = (ncol, nlay), (NBNDSW, ncol, nlay), (NGPTSW, ncol, nlay)
    ins = [_f(play, cl), _f(cldfrac, cl), _f(ciwp, cl), _f(clwp, cl), _f(rei, cl), _f(rel, cl),
           _f(tauc, bcl), _f(ssac, bcl), _f(asmc, bcl), _f(fsfc, bcl),
           _f(alpha if alpha is not None else np.zeros(cl), cl)]
    outs = [np.zeros(gcl, order="F") for _ in range(3)] + [np.zeros(cl, order="F") for _ in range(2)] + \
           [np.zeros(gcl, order="F") for _ in range(4)]
    _check(lib().mcica_subcol_sw_c(ncol, nlay, icld, permuteseed, irng, *[_p(x) for x in ins],
                                   *[_p(x) for x in outs]))
    return tuple(outs)


def mt_window(seed, offset):
    """The 624 raw MT19937 state words behind outputs ``offset`` ..
    ``offset + 623`` of the McICA generator seeded with ``seed``, computed on
    the host by jump-ahead (no GPU needed)."""
    w = np.zeros(624, dtype=np.uint32)
    _check(lib().rrtmg_sw_mt_window_c(seed, offset, w.ctypes.data_as(C.POINTER(C.c_uint32))))
    return w


def mt_temper(y):
    """MT19937 output tempering of raw state words (uint32 array)."""
    y = np.asarray(y, dtype=np.uint32).copy()
    y ^= y >> np.uint32(11)
    y ^= (y << np.uint32(7)) & np.uint32(0x9d2c5680)
    y ^= (y << np.uint32(15)) & np.uint32(0xefc60000)
    y ^= y >> np.uint32(18)
    return y


def mt_stream_dev(seed, n, out_ptr, log_seg=0, stream=0):
    """Outputs 0 .. n-1 of the MT19937 stream (tempered uint32) into the
    device buffer at ``out_ptr``, in segments of 2**log_seg words."""
    _check(lib().rrtmg_sw_mt_stream_dev_c(seed, n, C.c_void_p(out_ptr), log_seg, C.c_void_p(stream)))


def get_alpha(iplon, ncol, nlayers, icld, idcor, decorr_con, dz, lat, juldat, cldfrac):
    """get_alpha (mcica_subcol_gen_sw.f90:66-178); returns alpha (ncol, nlayers)."""
    cl = (ncol, nlayers)
    dz, lat, cldfrac = _f(dz, cl), _f(lat, (ncol,)), _f(cldfrac, cl)
    alpha = np.zeros(cl, order="F")
    _check(lib().get_alpha_c(ncol, nlayers, icld, idcor, C.c_double(decorr_con), _p(dz), _p(lat), juldat,
                             _p(cldfrac), _p(alpha)))
    return alpha


def rrtmg_sw_dev(args, stream=0, clouds=None):
    """Device-pointer entry point: ``args`` / ``clouds`` are filled
    :class:`RrtmgSwArgs` / :class:`RrtmgSwClouds` whose pointers are device
    addresses (e.g. from ``torch.Tensor.data_ptr()``)."""
    if clouds is None:
        _check(lib().rrtmg_sw_dev_c(C.byref(args), C.c_void_p(stream)))
    else:
        _check(lib().rrtmg_sw_mcica_dev_c(C.byref(args), C.byref(clouds), C.c_void_p(stream)))


AD_LAYER = ("tlay", "h2ovmr", "o3vmr", "clwp", "ciwp")
AD_SFC = ("asdir", "asdif", "aldir", "aldif")


def _ad_call(kw, clouds, weights, store, direction):
    ncol, nlay = kw["ncol"], kw["nlay"]
    cl, cl1 = (ncol, nlay), (ncol, nlay + 1)
    keep = {}
    a = RrtmgSwArgs()
    a.ncol, a.nlay, a.icld, a.iaer = ncol, nlay, kw["icld"], kw["iaer"]
    for name, shp in (("play", cl), ("plev", cl1), ("tlay", cl), ("h2ovmr", cl), ("o3vmr", cl), ("co2vmr", cl),
                      ("ch4vmr", cl), ("o2vmr", cl), ("asdir", (ncol,)), ("asdif", (ncol,)), ("aldir", (ncol,)),
                      ("aldif", (ncol,)), ("coszen", (ncol,)), ("tauaer", (ncol, nlay, NBNDSW)),
                      ("ssaaer", (ncol, nlay, NBNDSW)), ("asmaer", (ncol, nlay, NBNDSW)), ("ecaer", (ncol, nlay, 6))):
        keep[name] = _f(kw.get(name), shp)
        setattr(a, name, _p(keep[name]))
    a.adjes, a.dyofyr, a.scon, a.isolvar = kw["adjes"], kw["dyofyr"], kw["scon"], kw["isolvar"]
    a.inflgsw, a.iceflgsw, a.liqflgsw = kw["inflgsw"], kw["iceflgsw"], kw["liqflgsw"]
    a.idelm = 1
    c = None
    if clouds is not None:
        c = RrtmgSwClouds()
        c.permuteseed = clouds.get("permuteseed", NGPTSW)
        c.irng = clouds.get("irng", 0)
        for name, shp in (("cldfrac", cl), ("ciwp", cl), ("clwp", cl), ("rei", cl), ("rel", cl),
                          ("tauc", (NBNDSW, ncol, nlay)), ("ssac", (NBNDSW, ncol, nlay)),
                          ("asmc", (NBNDSW, ncol, nlay)), ("fsfc", (NBNDSW, ncol, nlay)), ("alpha", cl)):
            keep["c_" + name] = _f(clouds.get(name), shp)
            setattr(c, name, _p(keep["c_" + name]))
    d = RrtmgSwAdArgs()
    d.w_toa_up, d.w_sfc_net, d.w_hr_sum = weights
    d.store = -1 if store == "auto" else (1 if store else 0)
    out = {"J": np.zeros(ncol)}
    if direction is None:
        out.update({k: np.zeros(cl, order="F") for k in AD_LAYER})
        out.update({k: np.zeros(ncol) for k in AD_SFC})
        for k in AD_LAYER + AD_SFC:
            setattr(d, k, _p(out[k]))
    else:
        out["dJ"] = np.zeros(ncol)
        d.dJ = _p(out["dJ"])
        for k in AD_LAYER + AD_SFC:
            if direction.get(k) is not None:
                keep["dir_" + k] = _f(direction[k], cl if k in AD_LAYER else (ncol,))
                setattr(d, k, _p(keep["dir_" + k]))
    d.J = _p(out["J"])
    cp = C.byref(c) if c is not None else None
    if direction is None:
        _check(lib().rrtmg_sw_ad_c(C.byref(a), cp, C.byref(d)))
    else:
        _check(lib().rrtmg_sw_tl_c(C.byref(a), cp, C.byref(d)))
    return out


def rrtmg_sw_ad(kw, clouds=None, weights=(1.0, 0.0, 0.0), store=True):
    """Adjoint: J and its gradients (dict keyed by AD_LAYER + AD_SFC) for the
    objective J = w_toa_up*swuflx(top) + w_sfc_net*net flux(sfc) + w_hr_sum*sum(swhr);
    ``kw`` holds the rrtmg_sw arguments (as for :func:`rrtmg_sw`).  ``store``:
    True keeps the local Jacobians, False recomputes them, "auto" lets the
    library choose by free device memory."""
    return _ad_call(kw, clouds, weights, store, None)


def rrtmg_sw_tl(kw, direction, clouds=None, weights=(1.0, 0.0, 0.0)):
    """Tangent-linear: J and dJ along ``direction`` (dict keyed like the gradients)."""
    return _ad_call(kw, clouds, weights, True, direction)


def rrtmg_sw_static_dev(args, stream=0, clouds=None):
    """Allocation-free variant of :func:`rrtmg_sw_dev` for callers that may
    not allocate device memory while they run: the solve's scratch is a
    fixed 256 MiB area inside the library (one slot per SM must fit, else
    RRTMGError with code 5).  The first call per device looks the area up
    and should come before any stream capture; two of its solves must never
    be in flight at once."""
    cp = C.byref(clouds) if clouds is not None else None
    _check(lib().rrtmg_sw_static_dev_c(C.byref(args), cp, C.c_void_p(stream)))


class BatchPlan:
    """A planned batch of device-pointer instances (rrtmg_sw_batch_plan_c):
    ``args`` and ``clouds`` are lists of :class:`RrtmgSwArgs` /
    :class:`RrtmgSwClouds` (clouds may be None for an all-clear batch)."""

    def __init__(self, args, clouds=None, stream=0):
        n = len(args)
        self._a = (RrtmgSwArgs * n)(*args)
        self._c = None
        if clouds is not None:
            self._c = (RrtmgSwClouds * n)(*[c if c is not None else RrtmgSwClouds() for c in clouds])
        self.handle = C.c_void_p()
        _check(lib().rrtmg_sw_batch_plan_c(self._a, self._c, n, C.c_void_p(stream), C.byref(self.handle)))

    def run(self, stream=0):
        _check(lib().rrtmg_sw_batch_run_c(self.handle, C.c_void_p(stream)))

    def info(self):
        """The autotuner's choice and trials: grid, deepest_first, tile
        (columns, g-points per CTA), trial_ms and trials (tile columns,
        deepest first, CTAs per SM) in the same order."""
        cap = 64
        grid, desc, nt = C.c_int32(), C.c_int32(), C.c_int32(cap)
        ms = (C.c_float * cap)()
        _check(lib().rrtmg_sw_batch_info_c(self.handle, C.byref(grid), C.byref(desc), ms, C.byref(nt)))
        cols, gpts, nc = C.c_int32(), C.c_int32(), C.c_int32(cap)
        cfg = (C.c_int32 * cap)()
        _check(lib().rrtmg_sw_batch_tile_c(self.handle, C.byref(cols), C.byref(gpts), cfg, C.byref(nc)))
        trials = [(v >> 16, bool((v >> 8) & 255), v & 255) for v in cfg[:min(nc.value, cap)]]
        return {"grid": grid.value, "deepest_first": bool(desc.value), "tile": (cols.value, gpts.value),
                "trial_ms": list(ms[:min(nt.value, cap)]), "trials": trials}

    def close(self):
        if self.handle:
            lib().rrtmg_sw_batch_free_c(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def last_launch_count():
    return lib().rrtmg_sw_last_launch_count_c()


KERNEL_FP64, KERNEL_FP32, KERNEL_FP32_TILED = 0, 1, 2


def last_kernel():
    """Kernel of the most recent solve's main launch (KERNEL_*; -1 before any)."""
    return lib().rrtmg_sw_last_kernel_c()


def last_tile_slots():
    """Pair slots of the most recent solve's tiled kernel (3 or 2; 0: not tiled)."""
    return lib().rrtmg_sw_last_tile_slots_c()


def last_fp32_stats():
    """FP32 form's counters of the most recent solve: cells redone in FP64,
    of those past the scratch kernel's queue, column pairs the tiled kernel
    handed back, subcolumns the tiled kernel swept a second time."""
    out = (C.c_int64 * 4)()
    _check(lib().rrtmg_sw_last_fp32_stats_c(out))
    return dict(redone_cells=out[0], past_queue=out[1], pairs_handed_back=out[2], subcolumns_swept_twice=out[3])


def setcoef_indices(ncol, nlay, play, plev, tlay, h2ovmr, o3vmr, co2vmr, ch4vmr, o2vmr, **_):
    """setcoef_sw's indices (rrtmg_sw_setcoef.f90:158-200) as the solve kernels compute them:
    dict of jp, jt, jt1, indself, indfor (ncol, nlay) and laytrop (ncol), int32."""
    cl = (ncol, nlay)
    keep = [_f(play, cl), _f(plev, (ncol, nlay + 1)), _f(tlay, cl), _f(h2ovmr, cl), _f(o3vmr, cl),
            _f(co2vmr, cl), _f(ch4vmr, cl), _f(o2vmr, cl)]
    a = RrtmgSwArgs()
    a.ncol, a.nlay = ncol, nlay
    for k, v in zip(("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr"), keep):
        setattr(a, k, v.ctypes.data_as(_dp))
    outs = {k: np.zeros(cl, dtype=np.int32, order="F") for k in ("jp", "jt", "jt1", "indself", "indfor")}
    lt = np.zeros(ncol, dtype=np.int32)
    ip = lambda x: x.ctypes.data_as(C.POINTER(C.c_int32))
    _check(lib().rrtmg_sw_setcoef_c(C.byref(a), *[ip(outs[k]) for k in ("jp", "jt", "jt1", "indself", "indfor")],
                                    ip(lt)))
    outs["laytrop"] = lt
    return outs
