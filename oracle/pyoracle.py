"""ctypes binding of the FP64 CPU oracle (``liboracle_rrtmg_sw.so``).

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py as the oracle for the GPU library.  Nothing in
``rrtmg_sw_gb300`` imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_rrtmg_sw.so")
TABLES = os.path.join(os.path.dirname(HERE), "rrtmg_sw_gb300", "data", "rrtmg_sw_tables.bin")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class RrtmgSwArgs(C.Structure):
    """Mirror of ``orc_rrtmg_sw_args`` (field order of rrtmg_sw_rad.f90:99-111)."""
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


class ColumnCase(C.Structure):
    _fields_ = [
        ("nlay", C.c_int32), ("icld", C.c_int32), ("iaer", C.c_int32), ("idelm", C.c_int32),
        ("imca", C.c_int32), ("nmca", C.c_int32), ("idcor", C.c_int32), ("juldat", C.c_int32),
        ("inflag", C.c_int32), ("iceflag", C.c_int32), ("liqflag", C.c_int32), ("isolvar", C.c_int32),
        ("istart", C.c_int32), ("iend", C.c_int32),
        ("zenith", C.c_double), ("decorr_con", C.c_double), ("lat", C.c_double),
        ("svar_f", C.c_double), ("svar_s", C.c_double), ("svar_i", C.c_double),
        ("svar_f_bnd", _dp), ("svar_s_bnd", _dp), ("svar_i_bnd", _dp), ("adjflux", _dp),
        ("albedo", _dp),
        ("pavel", _dp), ("tavel", _dp), ("pz", _dp), ("tz", _dp), ("coldry", _dp),
        ("wkl", _dp), ("dz", _dp),
        ("cldfrac", _dp), ("ciwp", _dp), ("clwp", _dp), ("rei", _dp), ("rel", _dp),
        ("tauc", _dp), ("ssac", _dp), ("asmc", _dp), ("fsfc", _dp),
        ("tauaer", _dp), ("ssaaer", _dp), ("asmaer", _dp),
        ("uflx", _dp), ("dflx", _dp), ("dirdflx", _dp), ("difdflx", _dp), ("fnet", _dp), ("htr", _dp),
    ]


_lib = None


def build():
    """Compile the oracle with its Makefile (test infrastructure)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_init.argtypes = [C.c_char_p, C.c_double]
        L.orc_rrtmg_sw.argtypes = [C.POINTER(RrtmgSwArgs)]
        L.orc_rrtmg_sw_nomcica.argtypes = [C.POINTER(RrtmgSwArgs)] + [_dp] * 9
        L.orc_column_mode.argtypes = [C.POINTER(ColumnCase)]
        L.orc_get_alpha.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_int, _dp, _dp]
        L.orc_mcica_subcol_sw.argtypes = [C.c_int] * 5 + [_dp] * 11 + [_dp] * 9
        L.orc_mt_real.argtypes = [C.c_int, C.c_int, _dp]
        L.orc_kiss_real.argtypes = [C.c_int32] * 4 + [C.c_int, _dp]
        L.orc_setcoef_indices.argtypes = [C.c_int, _dp, _dp, _dp, _dp] + [_ip] * 6
        L.orc_gcm_setcoef_indices.argtypes = [C.c_int, C.c_int] + [_dp] * 9 + [_ip] * 6
        L.orc_exp_table.argtypes = [_dp]
        L.orc_heatfac.restype = C.c_double
        L.orc_solar_factors.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int] + [_dp] * 6
        rc = L.orc_init(TABLES.encode(), C.c_double(1.004e3))
        if rc != 0:
            raise RuntimeError("oracle init failed: %d" % rc)
        _lib = L
    return _lib


def init(cpdair):
    rc = lib().orc_init(TABLES.encode(), C.c_double(cpdair))
    if rc != 0:
        raise RuntimeError("oracle init failed: %d" % rc)


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def column_mode(case, istart=16, iend=29, nmca=200):
    """Run one golden column case (dict from tests/golden/std_atm_cases.json).

    Optional keys ``svar`` (f, s, i) and ``svar_bnd`` (3 x 14) carry the
    solar-variability factors of ``solar_factors``; both default to 1."""
    nlay = case["nlay"]
    keep = []

    def arr(x, n=None):
        a = _f64(x)
        if n is not None:
            assert a.size == n, (a.size, n)
        keep.append(a)
        return _p(a)

    ones = [1.0] * 14
    c = ColumnCase()
    c.nlay, c.icld, c.iaer, c.idelm = nlay, case["icld"], case["iaer"], case["idelm"]
    c.imca, c.nmca, c.idcor, c.juldat = case["imca"], nmca, case["idcor"], case["juldat"]
    c.inflag, c.iceflag, c.liqflag, c.isolvar = case["inflag"], case["iceflag"], case["liqflag"], case["isolvar"]
    c.istart, c.iend = istart, iend
    c.zenith, c.decorr_con, c.lat = case["zenith"], case["decorr_con"], case["lat"]
    c.svar_f, c.svar_s, c.svar_i = case.get("svar", (1.0, 1.0, 1.0))
    bnd = case.get("svar_bnd", (ones, ones, ones))
    c.svar_f_bnd, c.svar_s_bnd, c.svar_i_bnd = arr(bnd[0], 14), arr(bnd[1], 14), arr(bnd[2], 14)
    c.adjflux, c.albedo = arr(case["adjflux"], 14), arr(case["albedo"], 14)
    c.pavel, c.tavel = arr(case["pavel"], nlay), arr(case["tavel"], nlay)
    c.pz, c.tz = arr(case["pz"], nlay + 1), arr(case["tz"], nlay + 1)
    c.coldry, c.wkl, c.dz = arr(case["coldry"], nlay), arr(case["wkl"], 7 * nlay), arr(case["dz"], nlay)
    for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
        setattr(c, k, arr(case[k], nlay))
    z14 = np.zeros(14 * nlay)
    c.tauc, c.ssac, c.asmc, c.fsfc = arr(z14), arr(np.ones(14 * nlay)), arr(z14), arr(z14)
    for k in ("tauaer", "ssaaer", "asmaer"):
        setattr(c, k, arr(case.get(k, z14), 14 * nlay))
    out = {k: np.zeros(nlay + 1) for k in ("uflx", "dflx", "dirdflx", "difdflx", "fnet", "htr")}
    for k, v in out.items():
        setattr(c, k, _p(v))
    rc = lib().orc_column_mode(C.byref(c))
    if rc != 0:
        raise RuntimeError("orc_column_mode failed: %d" % rc)
    return out


def solar_factors(isolvar, scon, adjes=1.0, dyofyr=0, indsolvar=None, solcycfrac=None, bndsolvar=None):
    """Solar-variability factors of one solar record (``orc_solar_factors``):
    dict with svar (3), svar_bnd (3 x 14) and adjflux (14)."""
    keep = [None if x is None else _f64(np.atleast_1d(x)) for x in (indsolvar, solcycfrac, bndsolvar)]
    svar, bnd, adj = np.zeros(3), np.zeros(42), np.zeros(14)
    rc = lib().orc_solar_factors(isolvar, scon, adjes, dyofyr, *(_p(x) for x in keep), _p(svar), _p(bnd), _p(adj))
    if rc != 0:
        raise RuntimeError("orc_solar_factors failed: %d" % rc)
    return dict(svar=svar, svar_bnd=bnd.reshape(3, 14), adjflux=adj)


GCM_INPUTS = ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
              "asdir", "asdif", "aldir", "aldif", "coszen")
MCICA_INPUTS = ("cldfmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl")
AER_INPUTS = ("tauaer", "ssaaer", "asmaer", "ecaer")
EXTRA_OUTPUTS = ("dirdflux", "difdflux", "uvdflx", "nidflx", "dirdnuv", "difdnuv", "dirdnir", "difdnir")


NOMCICA_INPUTS = ("cldfr", "taucld", "ssacld", "asmcld", "fsfcld", "cicewp", "cliqwp", "reice", "reliq")


def rrtmg_sw(ncol, nlay, icld, iaer, inp, adjes=1.0, dyofyr=0, scon=1360.85, isolvar=0,
             inflgsw=2, iceflgsw=3, liqflgsw=1, idelm=1, nthreads=0, extra=False,
             bndsolvar=None, indsolvar=None, solcycfrac=None, nomcica=False, bands=False):
    """GCM entry point.  ``inp`` maps argument names to Fortran-ordered
    (column-major) FP64 arrays flattened to 1-D.  With ``nomcica=True`` the
    non-McICA rrtmg_sw runs on the NOMCICA_INPUTS arrays of ``inp``."""
    keep = []

    def arr(x):
        a = _f64(x).ravel(order="F")
        keep.append(a)
        return _p(a)

    a = RrtmgSwArgs()
    a.ncol, a.nlay, a.icld, a.iaer = ncol, nlay, icld, iaer
    for k in GCM_INPUTS:
        setattr(a, k, arr(inp[k]))
    a.adjes, a.dyofyr, a.scon, a.isolvar = adjes, dyofyr, scon, isolvar
    a.inflgsw, a.iceflgsw, a.liqflgsw = inflgsw, iceflgsw, liqflgsw
    zg = None
    for k in MCICA_INPUTS:
        if k in inp:
            setattr(a, k, arr(inp[k]))
        else:
            if zg is None:
                zg = np.zeros(112 * ncol * nlay)
                keep.append(zg)
            setattr(a, k, _p(zg))
    for k in AER_INPUTS:
        if k in inp:
            setattr(a, k, arr(inp[k]))
    out = {k: np.zeros(ncol * (nlay + 1)) for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    out.update({k: np.zeros(ncol * nlay) for k in ("swhr", "swhrc")})
    if extra:
        out.update({k: np.zeros(ncol * (nlay + 1)) for k in EXTRA_OUTPUTS})
    if bands:
        out.update({k: np.zeros(ncol * (nlay + 1) * 14) for k in ("bndfu", "bndfd", "bndfddir", "bndcu", "bndcd")})
    for k, v in out.items():
        setattr(a, k, _p(v))
    if bndsolvar is not None:
        a.bndsolvar = arr(bndsolvar)
    if indsolvar is not None:
        a.indsolvar = arr(indsolvar)
    if solcycfrac is not None:
        a.solcycfrac = arr([solcycfrac])
    a.idelm, a.nthreads = idelm, nthreads
    if nomcica:
        ptrs = [arr(inp[k]) if inp.get(k) is not None else None for k in NOMCICA_INPUTS]
        rc = lib().orc_rrtmg_sw_nomcica(C.byref(a), *ptrs)
    else:
        rc = lib().orc_rrtmg_sw(C.byref(a))
    if rc != 0:
        raise RuntimeError("orc_rrtmg_sw failed: %d" % rc)
    return out


def get_alpha(ncol, nlay, icld, idcor, decorr_con, dz, lat, juldat, cldfrac):
    dz, lat, cldfrac = _f64(dz), _f64(lat), _f64(cldfrac)
    alpha = np.zeros(ncol * nlay)
    rc = lib().orc_get_alpha(ncol, nlay, icld, idcor, decorr_con, _p(dz), _p(lat), juldat, _p(cldfrac), _p(alpha))
    if rc != 0:
        raise RuntimeError("orc_get_alpha failed: %d" % rc)
    return alpha


def mcica_subcol_sw(ncol, nlay, icld, permuteseed, irng, play, cldfrac, ciwp, clwp, rei, rel,
                    tauc, ssac, asmc, fsfc, alpha):
    ins = [_f64(x) for x in (play, cldfrac, ciwp, clwp, rei, rel, tauc, ssac, asmc, fsfc, alpha)]
    g = 112 * ncol * nlay
    outs = {k: np.zeros(g) for k in ("cldfmcl", "ciwpmcl", "clwpmcl")}
    outs["reicmcl"] = np.zeros(ncol * nlay)
    outs["relqmcl"] = np.zeros(ncol * nlay)
    outs.update({k: np.zeros(g) for k in ("taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")})
    order = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
    rc = lib().orc_mcica_subcol_sw(ncol, nlay, icld, permuteseed, irng, *[_p(x) for x in ins],
                                   *[_p(outs[k]) for k in order])
    if rc != 0:
        raise RuntimeError("orc_mcica_subcol_sw failed: %d" % rc)
    return outs


def mt_real(seed, n):
    out = np.zeros(n)
    lib().orc_mt_real(seed, n, _p(out))
    return out


def kiss_real(s1, s2, s3, s4, n):
    out = np.zeros(n)
    lib().orc_kiss_real(s1, s2, s3, s4, n, _p(out))
    return out


def setcoef_indices(pavel, tavel, coldry, wkl):
    nlay = len(pavel)
    outs = [np.zeros(nlay, dtype=np.int32) for _ in range(5)]
    lt = np.zeros(1, dtype=np.int32)
    ins = [_f64(x) for x in (pavel, tavel, coldry, wkl)]
    lib().orc_setcoef_indices(nlay, *[_p(x) for x in ins], *[o.ctypes.data_as(_ip) for o in outs],
                              lt.ctypes.data_as(_ip))
    return dict(zip(("jp", "jt", "jt1", "indself", "indfor"), outs), laytrop=int(lt[0]))


def gcm_setcoef_indices(kw):
    """setcoef_sw indices (jp, jt, jt1, indself, indfor: (ncol, nlay); laytrop: (ncol)) of the
    GCM-interface inputs in ``kw`` (rrtmg_sw keyword arrays), after inatm_sw's layer amounts."""
    ncol, nlay = kw["ncol"], kw["nlay"]
    ins = [_f64(np.asarray(kw[k]).ravel(order="F")) for k in
           ("play", "plev", "tlay", "h2ovmr", "co2vmr", "o3vmr", "n2ovmr", "ch4vmr", "o2vmr")]
    outs = [np.zeros(ncol * nlay, dtype=np.int32) for _ in range(5)]
    lt = np.zeros(ncol, dtype=np.int32)
    rc = lib().orc_gcm_setcoef_indices(ncol, nlay, *[_p(x) for x in ins], *[o.ctypes.data_as(_ip) for o in outs],
                                       lt.ctypes.data_as(_ip))
    assert rc == 0, rc
    res = {k: o.reshape((ncol, nlay), order="F") for k, o in zip(("jp", "jt", "jt1", "indself", "indfor"), outs)}
    res["laytrop"] = lt
    return res


def exp_table():
    out = np.zeros(10001)
    lib().orc_exp_table(_p(out))
    return out
