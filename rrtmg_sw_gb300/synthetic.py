"""Seeded synthetic GCM columns for tests and benchmarks.

Profiles follow the distributions used for the benchmark configurations:
surface pressure U(980,1030) hPa, log-spaced levels to 0.01 hPa with 2%
jitter, a standard-shaped temperature profile (288 K at the surface,
-6.5 K/km to 217 K at 11 km, isothermal to 20 km, +1 K/km to 48 km, then
decreasing to 190 K) plus N(0,5 K), water vapour U(0.2,1.5)e-2 exp(-z/2 km)
floored at 3e-6, ozone a Gaussian in ln p at 10 hPa with amplitude
U(6,9)e-6, fixed CO2/CH4/N2O/O2, albedos U(0.05,0.4) and coszen
U(0.05,1).  Optional cloud decks (a liquid deck in 850-600 hPa, an ice deck
in 400-200 hPa and a mixed deck in 600-400 hPa, 1-3 of them, each 2-6
layers thick, cloud fraction U(0.1,1), lognormal water paths with medians
50 (liquid) and 20 (ice) g m-2, rel U(5,20) um, rei U(20,80) um) and an
iaer=10 aerosol (tau 0.1 exp(-z/1.5 km) U(0.5,2) per band, ssa
U(0.85,0.99), asymmetry U(0.6,0.75)).  All arrays are FP64 in the
reference's Fortran shapes; layer 1 is at the surface.
"""
import numpy as np

RD, GRAV = 287.04, 9.80665


def _temperature(z_km):
    t = np.where(z_km <= 11.0, 288.0 - 6.5 * z_km, 216.5)
    t = np.where(z_km > 20.0, 216.5 + 1.0 * (z_km - 20.0), t)
    t = np.where(z_km > 48.0, np.maximum(244.5 - 2.8 * (z_km - 48.0), 190.0), t)
    return t


def make_columns(ncol, nlay, seed, clouds=False, aerosol=False, night_frac=0.0, lat=False, ptop=0.01):
    """Return a dict of GCM-interface inputs for ``ncol`` columns (top level at ``ptop`` hPa)."""
    rng = np.random.default_rng(seed)
    psfc = rng.uniform(980.0, 1030.0, ncol)
    frac = np.linspace(0.0, 1.0, nlay + 1)
    logp = np.log(psfc)[:, None] + frac[None, :] * (np.log(ptop) - np.log(psfc))[:, None]
    plev = np.exp(logp)
    jit = 1.0 + rng.uniform(-0.02, 0.02, (ncol, nlay + 1))
    jit[:, 0] = 1.0
    jit[:, -1] = 1.0
    plev = plev * jit
    plev = np.minimum.accumulate(plev, axis=1)  # strictly decreasing after the jitter
    play = np.sqrt(plev[:, :-1] * plev[:, 1:])
    # heights: scale-height first guess, then one hypsometric pass
    z_lev = 7.0 * np.log(psfc[:, None] / plev)
    z_lay = 0.5 * (z_lev[:, :-1] + z_lev[:, 1:])
    t_lay = _temperature(z_lay)
    dz = RD * t_lay / GRAV * np.log(plev[:, :-1] / plev[:, 1:]) / 1000.0
    z_lev = np.concatenate([np.zeros((ncol, 1)), np.cumsum(dz, axis=1)], axis=1)
    z_lay = 0.5 * (z_lev[:, :-1] + z_lev[:, 1:])
    tlay = _temperature(z_lay) + rng.normal(0.0, 5.0, (ncol, nlay))
    tlev = np.empty((ncol, nlay + 1))
    tlev[:, 1:-1] = 0.5 * (tlay[:, :-1] + tlay[:, 1:])
    tlev[:, 0] = tlay[:, 0]
    tlev[:, -1] = tlay[:, -1]
    tsfc = tlev[:, 0] + rng.normal(0.0, 2.0, ncol)
    h2o = rng.uniform(0.2, 1.5, (ncol, 1)) * 1.e-2 * np.exp(-z_lay / 2.0)
    h2o = np.maximum(h2o, 3.e-6)
    o3 = rng.uniform(6.0, 9.0, (ncol, 1)) * 1.e-6 * np.exp(-0.5 * (np.log(play / 10.0) / 1.2) ** 2)
    o3 = np.maximum(o3, 1.e-9)
    out = dict(
        play=play, plev=plev, tlay=tlay, tlev=tlev, tsfc=tsfc,
        h2ovmr=h2o, o3vmr=o3,
        co2vmr=np.full((ncol, nlay), 400.e-6), ch4vmr=np.full((ncol, nlay), 1.8e-6),
        n2ovmr=np.full((ncol, nlay), 3.2e-7), o2vmr=np.full((ncol, nlay), 0.209),
        asdir=rng.uniform(0.05, 0.4, ncol), asdif=rng.uniform(0.05, 0.4, ncol),
        aldir=rng.uniform(0.05, 0.4, ncol), aldif=rng.uniform(0.05, 0.4, ncol),
        coszen=rng.uniform(0.05, 1.0, ncol),
        dz=dz * 1000.0,
    )
    if night_frac > 0.0:
        night = rng.uniform(0.0, 1.0, ncol) < night_frac
        out["coszen"] = np.where(night, -rng.uniform(0.0, 1.0, ncol), out["coszen"])
    if lat:
        out["lat"] = rng.uniform(-90.0, 90.0, ncol)
    if clouds:
        cldfrac = np.zeros((ncol, nlay))
        ciwp = np.zeros((ncol, nlay))
        clwp = np.zeros((ncol, nlay))
        rel = np.zeros((ncol, nlay))
        rei = np.zeros((ncol, nlay))
        ndeck = rng.integers(1, 4, ncol)
        decks = ((850.0, 600.0, "liq"), (400.0, 200.0, "ice"), (600.0, 400.0, "mix"))
        for d, (pbot, ptop, kind) in enumerate(decks):
            use = ndeck > d
            thick = rng.integers(2, 7, ncol)
            # first layer inside the pressure band, at a random offset
            inband = (play <= pbot) & (play >= ptop)
            first = np.argmax(inband, axis=1)
            nin = inband.sum(axis=1)
            start = first + (rng.uniform(0, 1, ncol) * np.maximum(nin - 1, 1)).astype(int) * (nin > 1)
            cf = rng.uniform(0.1, 1.0, ncol)
            lw = np.exp(np.log(50.0) + 0.6 * rng.normal(size=ncol))
            iw = np.exp(np.log(20.0) + 0.6 * rng.normal(size=ncol))
            rl = rng.uniform(5.0, 20.0, ncol)
            ri = rng.uniform(20.0, 80.0, ncol)
            lay = np.arange(nlay)[None, :]
            mask = use[:, None] & (lay >= start[:, None]) & (lay < (start + thick)[:, None]) & (nin[:, None] > 0)
            cldfrac = np.where(mask, cf[:, None], cldfrac)
            if kind in ("liq", "mix"):
                clwp = np.where(mask, lw[:, None], clwp)
                rel = np.where(mask, rl[:, None], rel)
            if kind in ("ice", "mix"):
                ciwp = np.where(mask, iw[:, None], ciwp)
                rei = np.where(mask, ri[:, None], rei)
        # radii must be valid wherever a subcolumn may be cloudy
        rel = np.where(rel > 0.0, rel, 10.0)
        rei = np.where(rei > 0.0, rei, 50.0)
        out.update(cldfrac=cldfrac, ciwp=ciwp, clwp=clwp, rel=rel, rei=rei)
    if aerosol:
        base = 0.1 * np.exp(-z_lay / 1.5)
        tau = base[:, :, None] * rng.uniform(0.5, 2.0, (ncol, 1, 14))
        out.update(tauaer=tau, ssaaer=rng.uniform(0.85, 0.99, (ncol, nlay, 14)),
                   asmaer=rng.uniform(0.6, 0.75, (ncol, nlay, 14)))
    return out


def gcm_inputs(cols, icld=0, iaer=0, mcica=None):
    """Assemble the ``rrtmg_sw`` keyword arguments from ``make_columns``
    output plus optional subcolumn arrays ``mcica`` (9-tuple of
    mcica_subcol_sw)."""
    ncol, nlay = cols["play"].shape
    z = np.zeros((ncol, nlay))
    zg = np.zeros((112, ncol, nlay))
    kw = dict(ncol=ncol, nlay=nlay, icld=icld, iaer=iaer)
    for k in ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
              "asdir", "asdif", "aldir", "aldif", "coszen"):
        kw[k] = cols[k]
    kw.update(adjes=1.0, dyofyr=0, scon=1360.85, isolvar=0, inflgsw=2, iceflgsw=3, liqflgsw=1)
    if mcica is not None:
        names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
        kw.update(dict(zip(names, mcica)))
    else:
        kw.update(cldfmcl=zg, ciwpmcl=zg, clwpmcl=zg, reicmcl=z, relqmcl=z, taucmcl=zg, ssacmcl=zg + 1.0,
                  asmcmcl=zg, fsfcmcl=zg)
    zb = np.zeros((ncol, nlay, 14))
    kw.update(tauaer=cols.get("tauaer", zb), ssaaer=cols.get("ssaaer", zb + 1.0), asmaer=cols.get("asmaer", zb),
              ecaer=np.zeros((ncol, nlay, 6)))
    return kw
