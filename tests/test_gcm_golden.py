"""The reference's own example runs through the GCM entry points.

test_oracle_golden.py and test_rrtatm_golden.py pin the oracle's column mode
(the column driver's path, rrtmg_sw.1col.f90) to the printed tables of the
example runs.  Here the same runs go through the GCM call sequence,
get_alpha -> mcica_subcol_sw -> rrtmg_sw (rrtmg_sw_rad.f90:99-111), or the
non-McICA rrtmg_sw (rrtmg_sw_rad.nomcica.f90:97-109): the oracle's, and the
GPU library's FP64 form (print precision) and FP32 form (0.05 W m-2,
0.01 K/day), all 16 runs.

A column-driver case becomes GCM arguments as follows.
  - The driver takes column amounts (coldry, wkl in molecules cm-2), while
    inatm_sw derives them from each layer's pressure thickness,
    coldry = dp 1e3 N_A / (1e2 g amm (1 + h2o)) (rrtmg_sw_rad.f90:1550-1553),
    and wkl = coldry vmr.  The mixing ratios are wkl / coldry, and dp is
    chosen so that this formula returns the driver's coldry; plev is summed
    from the printed top level down.  plev enters the solve nowhere else but
    in the heating rate, so the heating rates are formed from the fluxes with
    the driver's own level pressures, htr(i-1) = (fnet(i) - fnet(i-1)) *
    heatfac / (pz(i-1) - pz(i)) (rrtmg_sw.1col.f90:811-821, 1799).
  - Albedo 1 - semiss: bands 16-24 and 29 take aldir/aldif, 25-28
    asdir/asdif (rrtmg_sw_rad.f90:673-683).  MLS-clr-sza65 gives a
    different albedo in each band: it runs once per band with that band's
    albedo everywhere and keeps that band's fluxes (the bands do not
    interact in the solve), its broadband fluxes summed over the bands.
  - McICA runs average 200 samples, sample ims drawn with the Mersenne
    Twister seeded (ims + 1) * 112 (mcica_subcol_gen_sw.1col.f90:255,
    rrtmg_sw.1col.f90:524); the samples are the columns of one call.  With
    idcor = 1 the driver sets juldat = 94 for get_alpha only.
  - Band blocks come from the per-band fluxes; direct and diffuse from the
    extra outputs.
"""
import json
import os

import numpy as np
import pytest

import pyoracle
import rrtatm

HERE = os.path.dirname(os.path.abspath(__file__))
STD = json.load(open(os.path.join(HERE, "golden", "std_atm_cases.json")))["cases"]
IATM1 = json.load(open(os.path.join(HERE, "golden", "std_atm_iatm1_cases.json")))["cases"]
TOL = {"uflx": 5e-5, "difdflx": 5e-5, "dirdflx": 5e-5, "dflx": 5e-5, "fnet": 5e-7, "htr": 5e-6}
TOL32 = {"uflx": 0.05, "difdflx": 0.05, "dirdflx": 0.05, "dflx": 0.05, "fnet": 0.05, "htr": 0.01}
NMCA = 200
# inatm_sw constants (rrtmg_sw_rad.f90:1520-1553)
AMD, AMW, AVOGAD, GRAV = 28.9660, 18.0160, 6.02214199e+23, 9.8066
UV = slice(9, 13)       # bands 25-28


def column_cases():
    """Column-driver cases (layers, solar settings, expected blocks) that map onto the GCM call."""
    out = [dict(c) for c in STD]
    for c in IATM1:
        d = dict(c)
        d["solar_record"] = True
        d.update(rrtatm.readprof_layers(c["atm"]))
        z = [0.0] * d["nlay"]
        d.update(cldfrac=z, ciwp=z, clwp=z, rei=z, rel=z, idcor=0, decorr_con=0.0, lat=0.0, inflag=0, iceflag=0,
                 liqflag=0)
        out.append(d)
    return out


CASES = column_cases()


def solar_args(case):
    """The solar record as the column driver maps it (rrtmg_sw.1col.f90:1391-1436)."""
    iso = case["isolvar"]
    kw = dict(isolvar=iso, scon=case.get("scon", 0.0), adjes=1.0, dyofyr=0)
    if case.get("solar_record"):
        sv = case["solvar"]
        if iso in (1, 2):
            kw["indsolvar"] = np.array(sv[:2])
        if iso == 1:
            kw["solcycfrac"] = case["solcycfrac"]
        if iso in (-1, 3):
            kw["bndsolvar"] = np.array(sv)
    return kw


def maps_albedo(case):
    """Whether the case's band albedos fit the GCM's near-IR / UV pair."""
    alb = np.array(case["albedo"])
    nir = np.concatenate([alb[:9], alb[13:]])
    return bool(np.all(nir == nir[0]) and np.all(alb[UV] == alb[UV][0]))


def gcm_arguments(case, ncol, albedo=None):
    """rrtmg_sw arguments (Fortran-ordered arrays) for ncol copies of one
    column-driver case; ``albedo`` replaces all four surface albedos."""
    nl = case["nlay"]
    pz = np.array(case["pz"])
    coldry = np.array(case["coldry"])
    wkl = np.array(case["wkl"]).reshape(nl, 7)
    vmr = wkl / coldry[:, None]
    h2o = vmr[:, 0]
    amm = (1.0 - h2o) * AMD + h2o * AMW
    dp = coldry * ((1.e2 * GRAV) * amm * (1.0 + h2o)) / (1.e3 * AVOGAD)
    plev = np.empty(nl + 1)
    plev[nl] = pz[nl]
    for l in range(nl - 1, -1, -1):
        plev[l] = plev[l + 1] + dp[l]
    alb = np.array(case["albedo"])
    if albedo is None:
        assert maps_albedo(case), "per-band albedo does not map"
        uv, nir = alb[UV][0], alb[0]
    else:
        uv = nir = albedo

    def cl(x):
        return np.tile(np.asarray(x, dtype=np.float64), (ncol, 1))

    def col(v):
        return np.full(ncol, float(v))

    tz = np.array(case["tz"])
    kw = dict(ncol=ncol, nlay=nl, icld=case["icld"], iaer=case["iaer"], play=cl(case["pavel"]), plev=cl(plev),
              tlay=cl(case["tavel"]), tlev=cl(tz), tsfc=col(tz[0]), h2ovmr=cl(vmr[:, 0]), o3vmr=cl(vmr[:, 2]),
              co2vmr=cl(vmr[:, 1]), ch4vmr=cl(vmr[:, 5]), n2ovmr=cl(vmr[:, 3]), o2vmr=cl(vmr[:, 6]),
              asdir=col(uv), asdif=col(uv), aldir=col(nir), aldif=col(nir),
              coszen=col(case["zenith"]), inflgsw=case["inflag"], iceflgsw=case["iceflag"],
              liqflgsw=case["liqflag"], idelm=case["idelm"])
    kw.update(solar_args(case))
    z14 = np.zeros((ncol, nl, 14))
    if case["iaer"] == 10:
        a = {k: np.asarray(case[k]).reshape(14, nl).T for k in ("tauaer", "ssaaer", "asmaer")}
        kw.update(tauaer=np.tile(a["tauaer"], (ncol, 1, 1)), ssaaer=np.tile(a["ssaaer"], (ncol, 1, 1)),
                  asmaer=np.tile(a["asmaer"], (ncol, 1, 1)))
    else:
        kw.update(tauaer=z14, ssaaer=z14 + 1.0, asmaer=z14)
    kw["ecaer"] = np.zeros((ncol, nl, 6))
    return kw


def mcica_samples(case, subcol, get_alpha):
    """McICA arrays of the NMCA samples, stacked as columns (G, NMCA, L) / (NMCA, L)."""
    nl = case["nlay"]
    alpha = np.zeros(nl)
    if case["icld"] in (4, 5):
        juldat = case["juldat"]
        if juldat == 0 and case["idcor"] == 1:
            juldat = 94
        alpha = get_alpha(case, juldat)
    names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
    acc = {k: [] for k in names}
    for ims in range(1, NMCA + 1):
        m = subcol(case, (ims + 1) * 112, alpha)
        for k in names:
            acc[k].append(np.asarray(m[k]))
    out = {}
    for k in names:
        if k in ("reicmcl", "relqmcl"):
            out[k] = np.stack([a.reshape(nl) for a in acc[k]])
        else:
            out[k] = np.stack([a.reshape(112, nl) for a in acc[k]], axis=1)
    return out


def blocks(case, res, heatfac, plev=None):
    """Printed quantities of every block from averaged GCM outputs (ncol samples).

    Heating rates are differenced from the fluxes with the driver's level
    pressures; with ``plev`` (the GCM levels of gcm_arguments) the broadband
    heating rate is instead the solver's own swhr scaled by the ratio of the
    two pressure thicknesses, below the top layer (rrtmg_sw sets the top
    layer's swhr to 0, rrtmg_sw_rad.f90:829-836), and band blocks carry no
    heating rate."""
    pz = np.array(case["pz"])
    pdp = pz[:-1] - pz[1:]
    got = {}
    for b in case["expected"]:
        band = b["istart"] == b["iend"]
        if band:
            ib = b["istart"] - 16
            u, d, dr = res["bndfu"][:, :, ib], res["bndfd"][:, :, ib], res["bndfddir"][:, :, ib]
        else:
            u, d, dr = res["swuflx"], res["swdflx"], res["dirdflux"]
        fn = d - u
        ht = np.zeros_like(fn)
        if plev is None:
            ht[:, :-1] = (fn[:, 1:] - fn[:, :-1]) * (heatfac / pdp)
        elif band:
            ht[:] = np.nan
        else:
            ht[:, :-1] = res["swhr"] * ((plev[:-1] - plev[1:]) / pdp)
            ht[:, -2] = np.nan
        n = u.shape[0]
        got[(b["istart"], b["iend"])] = dict(uflx=u.sum(0) / n, dflx=d.sum(0) / n, dirdflx=dr.sum(0) / n,
                                             difdflx=(d - dr).sum(0) / n, fnet=fn.sum(0) / n, htr=ht.sum(0) / n)
    return got


def run_case(case, run):
    """``run(case, albedo) -> (outputs, plev)`` once, or once per band when
    the albedos do not fit the GCM's pair: each band's fluxes from the run
    with its albedo, broadband fluxes summed over bands, no solver heating
    rate."""
    if maps_albedo(case):
        return run(case, None)
    res = None
    for ib, a in enumerate(case["albedo"]):
        r, plev = run(case, a)
        if res is None:
            res = {k: np.array(r[k]) for k in ("bndfu", "bndfd", "bndfddir")}
            res["swhr"] = np.full(np.shape(r["swhr"]), np.nan)
        for k in ("bndfu", "bndfd", "bndfddir"):
            res[k][:, :, ib] = r[k][:, :, ib]
    res["swuflx"] = res["bndfu"].sum(axis=2)
    res["swdflx"] = res["bndfd"].sum(axis=2)
    res["dirdflux"] = res["bndfddir"].sum(axis=2)
    return res, plev


def misses(case, got, tol):
    bad = []
    for b in case["expected"]:
        g = got[(b["istart"], b["iend"])]
        for k, t in tol.items():
            err = np.abs(g[k] - np.array(b[k]))
            err[np.isnan(err)] = 0.0
            bad += [(b["istart"], b["iend"], k, int(i), float(err[i])) for i in np.nonzero(err > t + 1e-9)[0]]
    return bad


# --- oracle -------------------------------------------------------------------------------------

def oracle_subcol(case, seed, alpha):
    nl = case["nlay"]
    z14 = np.zeros(14 * nl)
    m = pyoracle.mcica_subcol_sw(1, nl, case["icld"], seed, 1, *(np.asarray(case[k], dtype=np.float64) for k in
                                                                  ("pavel", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                 z14, z14 + 1.0, z14, z14, alpha)
    return {k: v.reshape((nl,) if k in ("reicmcl", "relqmcl") else (112, nl), order="F") for k, v in m.items()}


def oracle_alpha(case, juldat):
    nl = case["nlay"]
    return pyoracle.get_alpha(1, nl, case["icld"], case["idcor"], case["decorr_con"], np.asarray(case["dz"]),
                              np.array([case["lat"]]), juldat, np.asarray(case["cldfrac"], dtype=np.float64))


def fortran(x):
    return np.asarray(x, dtype=np.float64).ravel(order="F")


def oracle_run(case, albedo=None):
    ncol = NMCA if case["imca"] == 1 and case["icld"] >= 1 else 1
    kw = gcm_arguments(case, ncol, albedo)
    nl = case["nlay"]
    inp = {k: fortran(kw[k]) for k in pyoracle.GCM_INPUTS + pyoracle.AER_INPUTS}
    solar = {k: kw[k] for k in ("adjes", "dyofyr", "scon", "isolvar", "bndsolvar", "indsolvar", "solcycfrac")
             if k in kw}
    nomcica = case["icld"] >= 1 and case["imca"] == 0
    if ncol > 1:
        m = mcica_samples(case, oracle_subcol, oracle_alpha)
        inp.update({k: fortran(v) for k, v in m.items()})
    elif nomcica:
        t = np.asarray(case.get("tauc", np.zeros(14 * nl))).reshape(14, nl)
        inp.update(cldfr=fortran(case["cldfrac"]), cicewp=fortran(case["ciwp"]), cliqwp=fortran(case["clwp"]),
                   reice=fortran(case["rei"]), reliq=fortran(case["rel"]), taucld=fortran(t[:, None, :]),
                   ssacld=fortran(np.ones((14, 1, nl))), asmcld=fortran(np.zeros((14, 1, nl))),
                   fsfcld=fortran(np.zeros((14, 1, nl))))
    else:
        z = np.zeros(112 * nl)
        inp.update(cldfmcl=z, taucmcl=z, ssacmcl=z + 1.0, asmcmcl=z, fsfcmcl=z, ciwpmcl=z, clwpmcl=z,
                   reicmcl=np.zeros(nl), relqmcl=np.zeros(nl))
    out = pyoracle.rrtmg_sw(ncol, nl, case["icld"], case["iaer"], inp, inflgsw=kw["inflgsw"],
                            iceflgsw=kw["iceflgsw"], liqflgsw=kw["liqflgsw"], idelm=kw["idelm"], extra=True,
                            bands=True, nomcica=nomcica, **solar)
    res = {}
    for k in ("swuflx", "swdflx", "dirdflux"):
        res[k] = out[k].reshape((ncol, nl + 1), order="F")
    for k in ("bndfu", "bndfd", "bndfddir"):
        res[k] = out[k].reshape((ncol, nl + 1, 14), order="F")
    res["swhr"] = out["swhr"].reshape((ncol, nl), order="F")
    return res, kw["plev"][0]


@pytest.fixture(scope="module")
def heatfac():
    pyoracle.init(1.004e3)
    return pyoracle.lib().orc_heatfac()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_gcm_path(case, heatfac):
    res, plev = run_case(case, oracle_run)
    bad = misses(case, blocks(case, res, heatfac), TOL)
    assert not bad, bad[:10]
    # the solver's own heating rate, rescaled to the driver's pressure thicknesses
    bad = misses(case, blocks(case, res, heatfac, plev), TOL)
    assert not bad, bad[:10]


# --- GPU library --------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def gpu():
    from rrtmg_sw_gb300 import build, interface as gi
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    yield gi
    gi.set_form(gi.FORM_FP64)


def gpu_run(gi, case, albedo=None):
    ncol = NMCA if case["imca"] == 1 and case["icld"] >= 1 else 1
    kw = gcm_arguments(case, ncol, albedo)
    nl = case["nlay"]
    clouds = None
    nomcica = case["icld"] >= 1 and case["imca"] == 0
    if ncol > 1:
        def subcol(c, seed, alpha):
            z = np.zeros((14, 1, nl))
            names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl",
                     "fsfcmcl")
            m = gi.mcica_subcol_sw(1, 1, nl, c["icld"], seed, 1, *(np.asarray(c[k]).reshape(1, nl) for k in
                                                                   ("pavel", "cldfrac", "ciwp", "clwp", "rei",
                                                                    "rel")),
                                   z, z + 1.0, z, z, alpha.reshape(1, nl))
            return dict(zip(names, m))

        def alpha(c, juldat):
            return gi.get_alpha(1, 1, nl, c["icld"], c["idcor"], c["decorr_con"], np.asarray(c["dz"]).reshape(1, nl),
                                np.array([c["lat"]]), juldat, np.asarray(c["cldfrac"]).reshape(1, nl)).reshape(nl)

        kw.update(mcica_samples(case, subcol, alpha))
    else:
        z = np.zeros((112, ncol, nl))
        kw.update(cldfmcl=z, taucmcl=z, ssacmcl=z + 1.0, asmcmcl=z, fsfcmcl=z, ciwpmcl=z, clwpmcl=z,
                  reicmcl=np.zeros((ncol, nl)), relqmcl=np.zeros((ncol, nl)))
        if nomcica:
            t = np.asarray(case.get("tauc", np.zeros(14 * nl))).reshape(14, 1, nl)
            clouds = dict(cldfrac=np.asarray(case["cldfrac"]).reshape(1, nl),
                          ciwp=np.asarray(case["ciwp"]).reshape(1, nl), clwp=np.asarray(case["clwp"]).reshape(1, nl),
                          rei=np.asarray(case["rei"]).reshape(1, nl), rel=np.asarray(case["rel"]).reshape(1, nl),
                          tauc=t, ssac=np.ones((14, 1, nl)), asmc=np.zeros((14, 1, nl)), fsfc=np.zeros((14, 1, nl)))
    g = gi.rrtmg_sw(**kw, extra=True, bands=True, clouds=clouds, nomcica=nomcica)
    return {k: g[k] for k in ("swuflx", "swdflx", "dirdflux", "bndfu", "bndfd", "bndfddir", "swhr")}, kw["plev"][0]


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "fp32"])
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_gpu_gcm_path(gpu, form, case, heatfac):
    gpu.set_form(gpu.FORM_FP64 if form == "fp64" else gpu.FORM_FP32)
    try:
        res, plev = run_case(case, lambda c, a: gpu_run(gpu, c, a))
    finally:
        gpu.set_form(gpu.FORM_FP64)
    if form == "fp64":
        bad = misses(case, blocks(case, res, heatfac), TOL)
    else:
        # FP32 fluxes are rounded to ~1e-7 of their size, which a difference over a
        # 0.001 hPa layer turns into 0.1 K/day: the solver's own heating rate is checked
        bad = misses(case, blocks(case, res, heatfac, plev), TOL32)
    assert not bad, bad[:10]
