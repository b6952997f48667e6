"""Profile builder of the column driver's iatm = 1 input, restated for the oracle.

TEST INFRASTRUCTURE ONLY: used by tests/ to turn the records of the example
runs that take their layers from ``rrtatm.f`` into the layer inputs of the
oracle's column mode.  Nothing in ``rrtmg_sw_gb300`` imports this module.

With ``iatm = 1`` the column driver (``rrtmg_sw.1col.f90:1728-1768``) calls
``RRTATM`` (``rrtatm.f:5-205``), the LBLRTM atmosphere program, and reads
back its layer pressures, temperatures, level values and molecular column
amounts.  This module restates the part of that program an RRTM input can
reach: a user-supplied profile (``MODEL = 0``, unit codes 1-6 filled from
the built-in atmospheres) or one of the six built-in model atmospheres
(``MODEL`` 1-6, data extracted by oracle/extract_afgl.py); the vertical path
that ``ATMPTH`` forces (``ANGLE = 0``, ``rrtatm.f:787``); layer boundaries
given as altitudes or as pressures, with the hydrostatic altitudes of
``CMPALT`` for profiles on pressure levels and boundary pressures between
levels; and the refracted-ray integration of ``RFPATH``/``ALAYER`` with the
Curtis-Godson averages of ``FPACK``.  Everything else raises ``NotImplementedError``
(automatic layering, slant paths, trace species beyond the seventh from the
model atmospheres), never a silent approximation.  Arithmetic is IEEE double, as the reference is built
(``-r8``); sums run in the reference's order.
"""
import math

# physical constants passed to rrtatm.f through /CONSTS/ (rrtmg_sw.1col.f90:1339-1347,
# values of rrtmg_sw_init.f90:207-221)
PI = 2.0 * math.asin(1.0)
AVOGAD = 6.02214199e+23
ALOSMT = 2.6867775e+19
GASCON = 8.31447200e+07
# BLOCK DATA ATMCON (rrtatm.f:1728-1811)
PZERO, TZERO = 1013.25, 273.15
DELTAS = 5.0
KMXNOM = 7
AIRMWT = 28.964
AMWT = (18.015, 44.010, 47.998, 44.01, 28.011, 16.043, 31.999, 30.01, 64.06, 46.01, 17.03, 63.01, 17.00,
        20.01, 36.46, 80.92, 127.91, 51.45, 60.08, 30.03, 52.46, 28.014, 27.03, 50.49, 34.01, 26.03, 30.07,
        34.00, 66.01, 146.05, 34.08, 46.03, 33.00, 15.99, 98., 30.00, 97., 44.5, 32.04)
# WATVAP saturation density coefficients (rrtatm.f:3987-4120)
C1, C2, C3 = 18.9766, -14.9595, -2.4388
EPSILN = 1.0e-5     # ALAYER (rrtatm.f:5263-5505)
TOL = 5.0e-4        # AMERGE (rrtatm.f:5085-5262)
BIGNUM = 1.0e36     # RADRFD (rrtatm.f:7776-7799)


def _exp(x):
    try:
        return math.exp(x)
    except OverflowError:
        return math.inf


def jou(ch):
    """Unit code of one unit character (JOU, rrtatm.f:3400-3435)."""
    table = {"1": 1, "2": 2, "3": 3, "4": 4, "5": 5, "6": 6, " ": 10, "A": 10, "B": 11, "C": 12, "D": 13,
             "E": 14, "F": 15, "G": 16, "H": 17, "I": 18, "J": 19, "K": 20}
    if ch not in table:
        raise ValueError("JOU: BAD PARAM %r" % ch)
    return table[ch]


def check(a, ia, key):
    """Pressure / temperature unit conversion (CHECK, rrtatm.f:3436-3486)."""
    if ia <= 10:
        return a
    if key == 1:
        if ia == 11:
            return a * 1013.25
        if ia == 12:
            return a * 1013.25 / 760.0
        raise ValueError("CHECK(P)")
    if key == 2:
        if ia <= 11:
            return a + 273.15
        raise ValueError("CHECK(T)")
    raise ValueError("CHECK(R)")


def watvap(p, t, junit, wmol):
    """Water vapour number density in mol cm-3 (WATVAP, rrtatm.f:3987-4120)."""
    rhoair = ALOSMT * (p / PZERO) * (TZERO / t)
    a = TZERO / t
    b = AVOGAD / AMWT[0]
    r = AIRMWT / AMWT[0]

    def densat(atemp):
        return atemp * b * math.exp(C1 + C2 * atemp + C3 * atemp ** 2) * 1.0e-6

    if junit == 10:
        w = wmol * 1.0e-06
        return (w / (1. + w)) * rhoair
    if junit == 11:
        return wmol
    if junit == 12:
        w = wmol * r * 1.0e-3
        return (w / (1. + w)) * rhoair
    if junit == 13:
        return b * wmol * 1.0e-6
    if junit == 14:
        return ALOSMT * (wmol / PZERO) * (TZERO / t)
    if junit == 15:
        atd = TZERO / wmol
        return densat(atd) * wmol / t
    if junit == 16:
        atd = TZERO / (TZERO + wmol)
        return densat(atd) * (TZERO + wmol) / t
    if junit == 17:
        return densat(a) * (wmol / 100.0)
    raise ValueError("WATVAP: JUNIT %d" % junit)


def convrt(p, t, junit, wmol, nmol, co2mx):
    """Molecular number densities of one level (CONVRT, rrtatm.f:3875-3986)."""
    rhoair = ALOSMT * (p / PZERO) * (TZERO / t)
    den = [0.0] * nmol
    den[0] = watvap(p, t, junit[0], wmol[0])
    dryair = rhoair - den[0]
    for k in range(1, nmol):
        b = AVOGAD / AMWT[k]
        r = AIRMWT / AMWT[k]
        u = junit[k]
        if u <= 10:
            den[k] = wmol[k] * dryair * 1.e-6
        elif u == 11:
            den[k] = wmol[k]
        elif u == 12:
            den[k] = r * wmol[k] * 1.0e-3 * dryair
        elif u == 13:
            den[k] = b * wmol[k] * 1.0e-6
        elif u == 14:
            den[k] = ALOSMT * (wmol[k] / PZERO) * (TZERO / t)
        else:
            raise ValueError("CONVRT: JUNIT %d" % u)
    if co2mx > 0.:
        den[1] = co2mx * dryair * 1.e-06
    return den


_AFGL = None


def afgl():
    """The six built-in model atmospheres (rrtatm.f BLOCK DATA MLATMB,
    extracted by oracle/extract_afgl.py): alt (50), p and t (6 x 50), amol
    (6 x 8 x 50: ppmv of H2O, CO2, O3, N2O, CO, CH4, O2, then air cm-3)."""
    global _AFGL
    if _AFGL is None:
        import json
        import os
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "afgl_atmospheres.json")) as f:
            _AFGL = json.load(f)
    return _AFGL


def mdlatm_builtin(mdl, nmol, co2mx):
    """Levels of built-in model atmosphere ``mdl`` (MDLATM, rrtatm.f:2919-3047):
    water relative to the tabulated air density, the other species relative
    to dry air, CO2 scaled to co2mx ppmv when that is given."""
    if nmol > 7:
        raise NotImplementedError("trace species 8+ of the model atmospheres (/TRAC/) are not restated")
    d = afgl()
    m = mdl - 1
    co2rat = 1.
    if co2mx > 0.:
        co2rat = co2mx / 330.
    zmdl, pm, tm, denm = [], [], [], []
    for i in range(50):
        amol = [d["amol"][m][k][i] for k in range(8)]
        den1 = amol[0] * amol[7] * 1.0E-6
        dryair = amol[7] - den1
        den = [amol[k] * 1.0E-6 * dryair for k in range(nmol)]
        if nmol > 1:
            den[1] = den[1] * co2rat
        zmdl.append(d["alt"][i])
        pm.append(d["p"][m][i])
        tm.append(d["t"][m][i])
        denm.append(den)
    return zmdl, pm, tm, denm


def defalt(z, p, t, junitp, junitt, junit, wmol, nmol):
    """Values taken from a built-in model atmosphere for unit codes 1-6
    (DEFALT, rrtatm.f:3487-3680): 4-point Lagrange interpolation in altitude
    of ln p, t and the mixing ratios (ppmv), which then carry unit code 10.
    Returns (p, t, junit, wmol)."""
    d = afgl()
    alt = [None] + d["alt"]
    im50 = 50
    i2 = im50
    for im in range(2, im50 + 1):
        if alt[im] >= z:
            i2 = im
            break
    i1, i0, i3 = i2 - 1, i2 - 2, i2 + 1
    if i0 < 1:
        i0, i1, i2, i3 = i1, i2, i3, i3 + 1
    elif i3 > im50:
        if z > alt[im50]:
            raise ValueError("DEFAULT Z")
        i3, i2, i1 = i2, i1, i0
        i0 = i1 - 1
    z0, z1, z2, z3 = alt[i0], alt[i1], alt[i2], alt[i3]
    den1 = (z0 - z1) * (z0 - z2) * (z0 - z3)
    den2 = (z1 - z2) * (z1 - z3) * (z1 - z0)
    den3 = (z2 - z3) * (z2 - z0) * (z2 - z1)
    den4 = (z3 - z0) * (z3 - z1) * (z3 - z2)
    a1 = ((z - z1) * (z - z2) * (z - z3)) / den1
    a2 = ((z - z2) * (z - z3) * (z - z0)) / den2
    a3 = ((z - z3) * (z - z0) * (z - z1)) / den3
    a4 = ((z - z0) * (z - z1) * (z - z2)) / den4

    def val(x):
        return a1 * x[i0 - 1] + a2 * x[i1 - 1] + a3 * x[i2 - 1] + a4 * x[i3 - 1]

    if junitp <= 6:
        p = math.exp(val([math.log(v) for v in d["p"][junitp - 1]]))
    if junitt <= 6:
        t = val(d["t"][junitt - 1])
    junit, wmol = list(junit), list(wmol)
    for k in range(nmol):
        if junit[k] > 6:
            continue
        if k >= 7:
            raise NotImplementedError("trace species 8+ of the model atmospheres (/TRAC/) are not restated")
        wmol[k] = val(d["amol"][junit[k] - 1][k])
        junit[k] = 10
    return p, t, junit, wmol


def defalt_p(p, t, junitt, junit, wmol, nmol):
    """Unit codes 1-6 on a profile given on pressure levels (DEFALT_P,
    rrtatm.f:3681-3874): for each model, 4-point Lagrange interpolation in
    ln p on that model's own pressures of the temperature and mixing ratios
    (ppmv) that name it.  The pressure itself is kept.  Returns (t, junit, wmol)."""
    d = afgl()
    xlog_p = math.log(p)
    junit, wmol = list(junit), list(wmol)
    for j in range(1, 7):
        pm = [None] + d["p"][j - 1]
        lvl_50 = 50
        i2 = lvl_50
        for lvl in range(2, lvl_50 + 1):
            if p >= pm[lvl]:
                i2 = lvl
                break
        i1, i0, i3 = i2 - 1, i2 - 2, i2 + 1
        if i0 < 1:
            i0, i1, i2, i3 = i1, i2, i3, i3 + 1
        elif i3 > lvl_50:
            if p <= pm[lvl_50]:
                raise ValueError("DEFAULT P")
            i3, i2, i1 = i2, i1, i0
            i0 = i1 - 1
        p0, p1, p2, p3 = (math.log(pm[i]) for i in (i0, i1, i2, i3))
        den1 = (p0 - p1) * (p0 - p2) * (p0 - p3)
        den2 = (p1 - p2) * (p1 - p3) * (p1 - p0)
        den3 = (p2 - p3) * (p2 - p0) * (p2 - p1)
        den4 = (p3 - p0) * (p3 - p1) * (p3 - p2)
        a1 = ((xlog_p - p1) * (xlog_p - p2) * (xlog_p - p3)) / den1
        a2 = ((xlog_p - p2) * (xlog_p - p3) * (xlog_p - p0)) / den2
        a3 = ((xlog_p - p3) * (xlog_p - p0) * (xlog_p - p1)) / den3
        a4 = ((xlog_p - p0) * (xlog_p - p1) * (xlog_p - p2)) / den4

        def val(x):
            return a1 * x[i0 - 1] + a2 * x[i1 - 1] + a3 * x[i2 - 1] + a4 * x[i3 - 1]

        if junitt == j:
            t = val(d["t"][j - 1])
        for k in range(nmol):
            if junit[k] != j:
                continue
            if k >= 7:
                raise NotImplementedError("trace species 8+ of the model atmospheres (/TRAC/) are not restated")
            wmol[k] = val(d["amol"][j - 1][k])
            junit[k] = 10
    return t, junit, wmol


def cmpalt(pm, tm, denw, ref_z, ref_lat, re_):
    """Altitudes (km) of pressure levels by the hydrostatic equation with a
    moist-air compressibility factor (CMPALT, rrtatm.f:7800-7918): pm in mb,
    tm in K, denw the water vapour number densities, ref_z the first level's
    altitude, gravity at ref_lat falling off as (RE / (RE + z))**2."""
    ca0, ca1, ca2 = 1.58123E-6, -2.9331E-8, 1.1043E-10
    cb0, cb1 = 5.707E-6, -2.051E-8
    cc0, cc1 = 1.9898E-4, -2.376E-6
    cd, ce = 1.83E-11, -0.0765E-8
    xmass_h2o, xmass_dry = 0.018015, 0.0289654
    rgas, btz = 8.31441, 1.380662E-23
    n = len(pm)
    g0 = 9.80612 - 0.02586 * math.cos(2.0 * PI * ref_lat / 180.0)
    xmass_ratio = xmass_h2o / xmass_dry
    h2o_mixrat, comp_factor = [0.0] * n, [0.0] * n
    for j in range(n):
        dt = tm[j] - 273.15
        total_air = pm[j] * 1.0E-4 / (btz * tm[j])
        dry_air = total_air - denw[j]
        h2o_mixrat[j] = denw[j] / dry_air
        chim = xmass_ratio * h2o_mixrat[j]
        comp_factor[j] = (1. - (pm[j] * 100 / tm[j]) *
                          (ca0 + ca1 * dt + ca2 * dt ** 2 + (cb0 + cb1 * dt) * chim + (cc0 + cc1 * dt) * chim ** 2) +
                          (cd + ce * chim ** 2) * (pm[j] * 100. / tm[j]) ** 2)
    ztemp = [0.0] * n
    zmdl = [0.0] * n
    ztemp[0] = ref_z * 1000.0
    zmdl[0] = ref_z
    for i in range(n - 1):
        gave = g0 * (re_ / (re_ + ztemp[i] / 1000.0)) ** 2
        y = math.log(pm[i + 1] / pm[i])
        if y != 0.0:
            chi0 = h2o_mixrat[i]
            dchi = (h2o_mixrat[i + 1] - h2o_mixrat[i]) / y
            t0 = tm[i]
            dt = (tm[i + 1] - tm[i]) / y
            c1 = t0 + t0 * chi0
            c2 = t0 * dchi + dt * chi0 + dt
            c3 = dt * dchi
            b = 1 + xmass_ratio * chi0
            a = xmass_ratio * dchi
            alpha = a / b
            if abs(alpha * y) >= 0.01:
                raise ValueError("LAYER TOO THICK")
            xint_tot = c1 * y + 0.5 * (c2 - c1 * alpha) * y ** 2 + 0.3333 * (c3 - c2 * alpha + c1 * alpha ** 2) * y ** 3
            xint_tot = -xint_tot * rgas / (xmass_dry * gave * b)
            ztemp[i + 1] = ztemp[i] + xint_tot * comp_factor[i]
            zmdl[i + 1] = ztemp[i + 1] / 1000.
        else:
            ztemp[i + 1] = zmdl[i] * 1000.0
            zmdl[i + 1] = zmdl[i]
    return zmdl


def nsmdl(levels, nmol, co2mx, immax_b, ref_lat, re_):
    """User-supplied profile (NSMDL rrtatm.f:3048-3168, RDUNIT :3223-3399);
    a profile on pressure levels (IMMAX < 0) takes its altitudes from CMPALT,
    starting at the first level's altitude."""
    zmdl, pm, tm, denm = [], [], [], []
    for lv in levels:
        junitp, junitt = jou(lv["jcharp"]), jou(lv["jchart"])
        junit = [jou(c) for c in lv["jchar"][:nmol].ljust(nmol)]
        p = check(lv["p"], junitp, 1)
        t = check(lv["t"], junitt, 2)
        wmol = list(lv["wmol"][:nmol])
        if min([junitp, junitt] + junit) <= 6:
            if immax_b < 0:
                t, junit, wmol = defalt_p(p, t, junitt, junit, wmol, nmol)
            else:
                p, t, junit, wmol = defalt(lv["z"], p, t, junitp, junitt, junit, wmol, nmol)
        zmdl.append(lv["z"])
        pm.append(p)
        tm.append(t)
        denm.append(convrt(p, t, junit, wmol, nmol, co2mx))
    if immax_b < 0:
        zmdl = cmpalt(pm, tm, [d[0] for d in denm], zmdl[0], ref_lat, re_)
    for im in range(1, len(zmdl)):
        if zmdl[im] <= zmdl[im - 1]:
            raise ValueError("INPUT ALTITUDES NOT IN ASCENDING ORDER")
    return zmdl, pm, tm, denm


def expint(x1, x2, a):
    """Exponential interpolation (EXPINT, extra.f:223-244)."""
    if x1 == 0.0 or x2 == 0.0:
        return x1 + (x2 - x1) * a
    return x1 * (x2 / x1) ** a


def sclhtd(z1, z2, rfndx1, rfndx2):
    """Refractivity scale height and amplitude (SCLHTD, rrtatm.f:7717-7751)."""
    rf1 = rfndx1 + 1.0e-20
    rf2 = rfndx2 + 1.0e-20
    ratio = rf1 / rf2
    if abs(ratio - 1.0) < 1.0e-05:
        return 0.0, rfndx1
    return (z2 - z1) / math.log(ratio), rf1 * (rf2 / rf1) ** (-z1 / (z2 - z1))


def andexd(h, sh, gamma):
    """Refractive index (ANDEXD, rrtatm.f:7752-7775)."""
    if sh == 0.0:
        return 1.0 + gamma
    return 1.0 + gamma * _exp(-h / sh)


def radrfd(h, sh, gamma):
    """Radius of curvature of the ray (RADRFD, rrtatm.f:7776-7799)."""
    if sh == 0.0:
        return BIGNUM
    return sh * (1.0 + _exp(h / sh) / gamma)


class _Atm:
    """The profile and path state that rrtatm.f keeps in /CMN/, /DEAMT/ and /PARMTR/.

    Arrays are 1-based (index 0 unused) so the loops read as the reference's."""

    def __init__(self, zmdl, pm, tm, denm, nmol, re_):
        self.nmol = nmol
        self.re = re_
        self.deg = 180.0 / PI
        self.gcair = 1.0e-3 * GASCON / AVOGAD
        self.zmdl = [None] + list(zmdl)
        self.pm = [None] + list(pm)
        self.tm = [None] + list(tm)
        self.denm = [None] + [list(d) for d in denm]
        self.immax = len(zmdl)
        self.rfndxm = [None] * (self.immax + 1)

    def fndshd(self, h):
        """FNDSHD (rrtatm.f:7670-7716)."""
        i2 = self.immax
        for im in range(2, self.immax + 1):
            if self.zmdl[im] >= h:
                i2 = im
                break
        i1 = i2 - 1
        return sclhtd(self.zmdl[i1], self.zmdl[i2], self.rfndxm[i1], self.rfndxm[i2])


def _pressure_to_altitude(a, pval, ref_lat):
    """Altitude and temperature of a boundary given as a pressure (ATMPTH
    loop 160 and its H1/H2 twins, rrtatm.f:872-1080).  Between two profile
    levels the altitude blends the log-pressure interpolation with a CMPALT
    step from the level below, weighted by the cube of the log-pressure
    fraction."""
    lip = a.immax
    for cand in range(2, a.immax + 1):
        if pval > a.pm[cand]:
            lip = cand
            break
    if pval == a.pm[lip - 1]:
        return a.zmdl[lip - 1], a.tm[lip - 1]
    if pval == a.pm[lip]:
        return a.zmdl[lip], a.tm[lip]
    lpm = math.log(a.pm[lip] / a.pm[lip - 1])
    lp = math.log(pval / a.pm[lip - 1])
    hip = (a.zmdl[lip] - a.zmdl[lip - 1]) / lpm
    zint = a.zmdl[lip - 1] + hip * lp
    tip = (a.tm[lip] - a.tm[lip - 1]) / lpm
    t2 = a.tm[lip - 1] + tip * lp
    wvip = (a.denm[lip][0] - a.denm[lip - 1][0]) / lpm
    wv2 = a.denm[lip - 1][0] + wvip * lp
    z2 = cmpalt([a.pm[lip - 1], pval], [a.tm[lip - 1], t2], [a.denm[lip - 1][0], wv2], a.zmdl[lip - 1], ref_lat,
                a.re)[1]
    ratp = lp / lpm
    w = ratp ** 3
    return w * zint + (1 - w) * z2, t2


def _amerge(a, h1, h2, hmin, len_, zbnd):
    """Path levels: profile levels merged with layer boundaries (AMERGE, rrtatm.f:5085-5262)."""
    if len_ != 0:
        raise NotImplementedError("tangent paths (LEN = 1) are not restated")
    ibmax = len(zbnd) - 1
    hmid = min(h1, h2)
    hmax = max(h1, h2)
    ihmax = 2
    zh = [None, hmin, hmax, None]
    zout = [None, zh[1]]
    i1 = ibmax
    for i in range(1, ibmax + 1):
        if abs(zbnd[i] - zh[1]) < TOL:
            zh[1] = zbnd[i]
        if zbnd[i] > zh[1]:
            i1 = i
            break
    iout, ib, ih = 1, i1, 2
    while True:
        iout += 1
        zout.append(None)
        if ib <= ibmax:
            if abs(zbnd[ib] - zh[ih]) < TOL:
                zh[ih] = zbnd[ib]
            if zbnd[ib] < zh[ih]:
                zout[iout] = zbnd[ib]
                ib += 1
                continue
            if zbnd[ib] == zh[ih]:
                ib += 1
        zout[iout] = zh[ih]
        ih += 1
        if ih > ihmax:
            break
    ioutmx = iout

    im = None
    for cand in range(1, a.immax + 1):
        if a.zmdl[cand] >= hmin:
            im = cand
            break
    if im is None:
        raise ValueError("AMERGE - HMIN")
    n = a.nmol
    zpth, pp, tp, rfndxp, denp = [None], [None], [None], [None], [None]
    iphmid = 0
    ip = 0
    iout = 1
    while True:
        ip += 1
        interp = im > a.immax
        if not interp:
            if abs(zout[iout] - a.zmdl[im]) < TOL:
                a.zmdl[im] = zout[iout]
            interp = zout[iout] < a.zmdl[im]
        if not interp:
            if zout[iout] == a.zmdl[im]:
                iout += 1
            zpth.append(a.zmdl[im])
            pp.append(a.pm[im])
            tp.append(a.tm[im])
            rfndxp.append(a.rfndxm[im])
            denp.append(list(a.denm[im]))
            im += 1
            if abs(zpth[ip] - hmid) < TOL:
                hmid = zpth[ip]
            if zpth[ip] == hmid:
                iphmid = ip
            if abs(zpth[ip] - zout[ioutmx]) < TOL:
                zout[ioutmx] = zpth[ip]
            if zpth[ip] == zout[ioutmx]:
                break
            continue
        jm = max(im, 2)
        if jm > a.immax:
            raise ValueError("AMERGE: path above the profile")
        z = zout[iout]
        f = (z - a.zmdl[jm - 1]) / (a.zmdl[jm] - a.zmdl[jm - 1])
        zpth.append(z)
        pp.append(expint(a.pm[jm - 1], a.pm[jm], f))
        tp.append(a.tm[jm - 1] + (a.tm[jm] - a.tm[jm - 1]) * f)
        rfndxp.append(expint(a.rfndxm[jm - 1], a.rfndxm[jm], f))
        denp.append([expint(a.denm[jm - 1][k], a.denm[jm][k], f) for k in range(n)])
        if abs(zpth[ip] - hmid) < TOL:
            zpth[ip] = hmid
        if zpth[ip] == hmid:
            iphmid = ip
        iout += 1
        if abs(zpth[ip] - zout[ioutmx]) < TOL:
            zpth[ip] = zout[ioutmx]
        if zpth[ip] == zout[ioutmx]:
            break
    return dict(zout=zout, ioutmx=ioutmx, zpth=zpth, pp=pp, tp=tp, rfndxp=rfndxp, denp=denp, ipmax=ip,
                iphmid=iphmid)


def _alayer(a, path, j, sinai, cosai, cpath, sh, gamma):
    """Ray through path layer j with its absorber integrals (ALAYER, rrtatm.f:5263-5505)."""
    zpth, pp, tp, denp = path["zpth"], path["pp"], path["tp"], path["denp"]
    n = a.nmol
    z1 = zpth[j]
    z2 = zpth[j + 1]
    h1 = z1
    r1 = a.re + h1
    dhmin = DELTAS ** 2 / (2.0 * r1)
    sinai1 = sinai
    cosai1 = cosai
    if (1.0 - sinai) < EPSILN:
        raise NotImplementedError("near-horizontal rays are not restated")
    x1 = -r1 * cosai1
    ratio1 = r1 / radrfd(h1, sh, gamma)
    dsdx1 = 1.0 / (1.0 - ratio1 * sinai1 ** 2)
    dbndx1 = dsdx1 * sinai1 * ratio1 / r1
    s = 0.0
    bend = 0.0
    pa = pp[j]
    pb = pp[j + 1]
    if pb == pa:
        raise ValueError("LBLATM: PRESSURES IN ADJOINING LAYERS MUST DIFFER")
    ta = tp[j]
    tb = tp[j + 1]
    rhoa = pa / (a.gcair * ta)
    rhob = pb / (a.gcair * tb)
    dz = zpth[j + 1] - zpth[j]
    hp = -dz / math.log(pb / pa)
    if abs(rhob / rhoa - 1.0) >= EPSILN:
        hrho = -dz / math.log(rhob / rhoa)
    else:
        hrho = 1.0e30
    dena = list(denp[j])
    denb = list(denp[j + 1])
    hden = [0.0] * n
    for k in range(n):
        if (dena[k] == 0.0 or denb[k] == 0.0) or abs(1.0 - dena[k] / denb[k]) <= EPSILN:
            hden[k] = 0.0
        else:
            hden[k] = -dz / math.log(denb[k] / dena[k])
    ppsum = tpsum = rhopsm = 0.0
    amtp = [0.0] * n
    while True:
        dh = -DELTAS * cosai1
        dh = max(dh, dhmin)
        h3 = h1 + dh
        if h3 > z2:
            h3 = z2
        dh = h3 - h1
        r3 = a.re + h3
        h2 = h1 + dh / 2.0
        r2 = a.re + h2
        sinai2 = cpath / (andexd(h2, sh, gamma) * r2)
        sinai3 = cpath / (andexd(h3, sh, gamma) * r3)
        ratio2 = r2 / radrfd(h2, sh, gamma)
        ratio3 = r3 / radrfd(h3, sh, gamma)
        if (1.0 - sinai2) <= EPSILN:
            raise NotImplementedError("near-horizontal rays are not restated")
        cosai2 = -math.sqrt(1.0 - sinai2 ** 2)
        cosai3 = -math.sqrt(1.0 - sinai3 ** 2)
        x2 = -r2 * cosai2
        x3 = -r3 * cosai3
        d31 = x3 - x1
        d32 = x3 - x2
        d21 = x2 - x1
        if d32 == 0.0 or d21 == 0.0:
            w1 = 0.5 * d31
            w2 = 0.0
            w3 = 0.5 * d31
        else:
            w1 = (2.0 - d32 / d21) * d31 / 6.0
            w2 = d31 ** 3 / (d32 * d21 * 6.0)
            w3 = (2.0 - d21 / d32) * d31 / 6.0
        dsdx2 = 1.0 / (1.0 - ratio2 * sinai2 ** 2)
        dsdx3 = 1.0 / (1.0 - ratio3 * sinai3 ** 2)
        dbndx2 = dsdx2 * sinai2 * ratio2 / r2
        dbndx3 = dsdx3 * sinai3 * ratio3 / r3
        ds = w1 * dsdx1 + w2 * dsdx2 + w3 * dsdx3
        s = s + ds
        dbend = w1 * dbndx1 + w2 * dbndx2 + w3 * dbndx3
        bend = bend + dbend
        dsdz = ds / dh
        pb = pa * math.exp(-dh / hp)
        rhob = rhoa * math.exp(-dh / hrho)
        if (dh / hrho) >= EPSILN:
            ppsum = ppsum + dsdz * (hp / (1.0 + hp / hrho)) * (pa * rhoa - pb * rhob)
            tpsum = tpsum + dsdz * hp * (pa - pb) / a.gcair
            rhopsm = rhopsm + dsdz * hrho * (rhoa - rhob)
        else:
            ppsum = ppsum + 0.5 * ds * (pa * rhoa + pb * rhob)
            tpsum = tpsum + 0.5 * ds * (pa + pb) / a.gcair
            rhopsm = rhopsm + 0.5 * ds * (rhoa + rhob)
        for k in range(n):
            if hden[k] == 0.0 or abs(dh / hden[k]) < EPSILN:
                denb[k] = denp[j][k] + (denp[j + 1][k] - denp[j][k]) * (h3 - z1) / dz
                amtp[k] = amtp[k] + 0.5 * (dena[k] + denb[k]) * ds * 1.0e5
            else:
                denb[k] = denp[j][k] * math.exp(-(h3 - z1) / hden[k])
                amtp[k] = amtp[k] + dsdz * hden[k] * (dena[k] - denb[k]) * 1.0e5
        pa = pb
        rhoa = rhob
        dena = list(denb)
        if h3 < z2:
            h1 = h3
            r1 = r3
            sinai1 = sinai3
            ratio1 = ratio3
            cosai1 = cosai3
            x1 = x3
            dsdx1 = dsdx3
            dbndx1 = dbndx3
        else:
            return dict(sinai=sinai3, cosai=cosai3, s=s, bend=bend, ppsum=ppsum, tpsum=tpsum, rhopsm=rhopsm,
                        amtp=amtp)


def atmpth(atm):
    """Layers of one RRTM iatm = 1 input (ATMPTH, rrtatm.f:206-1727, ITYPE 2).

    ``atm`` holds the parsed records 3.1-3.5 (see tests/golden/make_golden.py).
    Returns the /PROFILE/ and /SPECIES/ contents: 1-based lists pbar, tbar,
    amount[k] (k = 0..nmol-1), wn2l, coldry and 0-based pz, tz, altz."""
    # record 3.1 and the defaults RRTM forces (:576-620)
    model = atm["model"]
    ibmax_b = atm["ibmax_b"]
    ibmax = abs(ibmax_b)
    nmol = atm["nmol"] or KMXNOM
    nozero = 1
    xvbar = 1.0
    if not 0 <= model <= 6:
        raise ValueError("CARD 3.1: MODEL out of range")
    re_ = atm["re"]
    if re_ == 0.0:
        re_ = {1: 6378.39, 4: 6356.91, 5: 6356.91}.get(model, 6371.23)
    hspace = atm["hspace"] if atm["hspace"] != 0. else 100.
    # record 3.2 (:786-795): RRTM sets ANGLE = 0
    h1, h2 = atm["h1"], atm["h2"]
    angle = 0.0
    range_, beta = atm["range"], atm["beta"]
    if ibmax == 0:
        raise NotImplementedError("automatic layering (AUTLAY) is not restated")
    bnd = atm["bnd"][:ibmax]
    if ibmax_b > 0 and any(bnd[i] <= bnd[i - 1] for i in range(1, ibmax)):
        raise ValueError("ZBND not ascending")
    if ibmax_b < 0 and any(bnd[i] >= bnd[i - 1] for i in range(1, ibmax)):
        raise ValueError("PBND not descending")
    # MDLATM (rrtatm.f:2919-3047) with the user profile of NSMDL
    ref_lat = atm["ref_lat"] if atm["ref_lat"] != 0 else 45.
    if model == 0:
        zmdl, pm, tm, denm = nsmdl(atm["levels"], nmol, atm["co2mx"], atm["immax_b"], ref_lat, re_)
    else:
        zmdl, pm, tm, denm = mdlatm_builtin(model, nmol, atm["co2mx"])
    ispace = 1
    for i, z in enumerate(zmdl):
        if hspace + 0.001 > z:
            ispace = i + 1
    zmdl, pm, tm, denm = zmdl[:ispace], pm[:ispace], tm[:ispace], denm[:ispace]
    a = _Atm(zmdl, pm, tm, denm, nmol, re_)
    zmax = a.zmdl[a.immax]
    # layer boundaries and path ends given as pressures (:866-1080)
    if ibmax_b < 0:
        zbnd = [None] + [_pressure_to_altitude(a, p, ref_lat)[0] for p in bnd]
        h1 = _pressure_to_altitude(a, h1, ref_lat)[0]
        h2 = _pressure_to_altitude(a, h2, ref_lat)[0]
        if h1 < 0.0 or h2 < 0.0:
            raise ValueError("COMPUTED ALTITUDE VALUE OF H1/H2 IS NEGATIVE")
    else:
        zbnd = [None] + list(bnd)
    if zbnd[1] < a.zmdl[1]:
        if abs(zbnd[1] - a.zmdl[1]) <= 0.0001:
            zbnd[1] = a.zmdl[1]
        else:
            raise ValueError("BOUNDARIES OUTSIDE OF ATMOS")
    # LOWTRAN6 refractive index (loop 170, :1093-1099)
    for im in range(1, a.immax + 1):
        pph2o = a.denm[im][0] * PZERO * a.tm[im] / (TZERO * ALOSMT)
        a.rfndxm[im] = ((83.42 + (185.08 / (1.0 - (xvbar / 1.14E+5) ** 2)) +
                         (4.11 / (1.0 - (xvbar / 6.24E+4) ** 2))) * (a.pm[im] * 288.15) /
                        (1013.25 * a.tm[im]) - (43.49 - (xvbar / 1.7E+4) ** 2) * (pph2o / 1013.25)) * 1.0E-06
    # FSCGEO (rrtatm.f:4121-4429), ITYPE 2 with RANGE = BETA = 0, and FNDHMN (:4655-4780)
    if range_ > 0.0 or beta > 0.0:
        raise NotImplementedError("slant paths given by RANGE or BETA are not restated")
    if h1 >= h2:
        raise ValueError("FSCGEO: H1 >= H2 with ANGLE = 0")
    sh, gamma = a.fndshd(h1)
    cpath = (a.re + h1) * andexd(h1, sh, gamma) * math.sin(angle / a.deg)
    sh, gamma = a.fndshd(h2)
    ch2 = (a.re + h2) * andexd(h2, sh, gamma)
    if abs(cpath / ch2) > 1.0:
        raise ValueError("FSCGEO: impossible geometry")
    hmin, len_ = h1, 0
    if hmin >= zmax:
        raise ValueError("FSCGEO: HMIN >= ZMAX")
    if h1 > zmax or h2 > zmax:
        raise NotImplementedError("paths above the profile (REDUCE) are not restated")
    # RFPATH (rrtatm.f:4892-5084), IORDER = 1, LEN = 0
    path = _amerge(a, h1, h2, hmin, len_, zbnd)
    sh, gamma = a.fndshd(h1)
    cpath = (a.re + h1) * andexd(h1, sh, gamma) * math.sin(angle / a.deg)
    if angle <= 45.0:
        sinai = math.sin(angle / a.deg)
        cosai = -math.cos(angle / a.deg)
    else:
        sinai = math.cos((90.0 - angle) / a.deg)
        cosai = -math.sin((90.0 - angle) / a.deg)
    layers = [None]
    for j in range(1, path["ipmax"]):
        sh, gamma = sclhtd(path["zpth"][j], path["zpth"][j + 1], path["rfndxp"][j], path["rfndxp"][j + 1])
        lay = _alayer(a, path, j, sinai, cosai, cpath, sh, gamma)
        sinai, cosai = lay["sinai"], lay["cosai"]
        layers.append(lay)
    # FPACK (rrtatm.f:5815-5992), NOZERO = 1
    zout, ioutmx, zpth, pp, tp = path["zout"], path["ioutmx"], path["zpth"], path["pp"], path["tp"]
    nl = ioutmx - 1
    pbar = [0.0] * (nl + 2)
    tbar = [0.0] * (nl + 2)
    rhosum = [0.0] * (nl + 2)
    amount = [[0.0] * (nl + 2) for _ in range(nmol)]
    pz = [0.0] * (nl + 1)
    tz = [0.0] * (nl + 1)
    pz[0], tz[0] = pp[1], tp[1]
    iout = 1
    for ip in range(1, path["ipmax"]):
        lay = layers[ip]
        pbar[iout] = pbar[iout] + lay["ppsum"]
        tbar[iout] = tbar[iout] + lay["tpsum"]
        rhosum[iout] = rhosum[iout] + lay["rhopsm"]
        for k in range(nmol):
            amount[k][iout] = amount[k][iout] + lay["amtp"][k]
        if iout + 1 <= ioutmx and zpth[ip + 1] == zout[iout + 1]:
            pz[iout] = pp[ip + 1]
            tz[iout] = tp[ip + 1]
            iout = iout + 1
    if iout != ioutmx:
        raise ValueError("ERROR FPACK")
    assert nozero == 1
    wn2l = [0.0] * (nl + 1)
    altz = [zout[1]] + [zout[l + 1] for l in range(1, nl + 1)]
    for l in range(1, nl + 1):
        pbar[l] = pbar[l] / rhosum[l]
        tbar[l] = tbar[l] / rhosum[l]
        rhosum[l] = rhosum[l] * 1.0E+5
        sumamt = 0.
        for k in range(nmol):
            sumamt = sumamt + amount[k][l]
        wn2l[l] = rhosum[l] - sumamt
    # punched layer amounts below one molecule cm-2 become zero (loop 277, :1385-1389)
    if atm["ipunch"] == 1 and atm["munits"] != 1:
        for l in range(1, nl + 1):
            for k in range(nmol):
                if amount[k][l] < 1.:
                    amount[k][l] = 0.0
    # dry air column (loop 285, :1415-1420)
    coldry = [0.0] * (nl + 1)
    for l in range(1, nl + 1):
        drair = wn2l[l]
        for m in range(1, nmol):
            drair = drair + amount[m][l]
        coldry[l] = drair
    return dict(nlayrs=nl, nmol=nmol, pbar=pbar[:nl + 1], tbar=tbar[:nl + 1], pz=pz, tz=tz, altz=altz,
                amount=[am[:nl + 1] for am in amount], wn2l=wn2l, coldry=coldry)


def readprof_layers(atm):
    """What readprof passes on for iatm = 1 (rrtmg_sw.1col.f90:1728-1768,
    1795-1812): layers surface-first, column amounts in molecules cm-2."""
    r = atmpth(atm)
    nl, nmol = r["nlayrs"], r["nmol"]
    wkl = [[r["amount"][m][l] for m in range(nmol)] for l in range(1, nl + 1)]
    wbrodl = [r["wn2l"][l] for l in range(1, nl + 1)]
    imix = 1
    for m in range(nmol):
        if wkl[0][m] > 1.0:
            imix = 0
            break
    coldry = []
    for l in range(nl):
        summol = 0.0
        for imol in range(1, nmol):
            summol = summol + wkl[l][imol]
        if imix == 1:
            cd = wbrodl[l] / (1.0 - summol)
            wkl[l] = [cd * w for w in wkl[l]]
        else:
            cd = wbrodl[l] + summol
        coldry.append(cd)
    wkl7 = [(row + [0.0] * 7)[:7] for row in wkl]
    return dict(nlay=nl, pavel=r["pbar"][1:], tavel=r["tbar"][1:], pz=list(r["pz"]), tz=list(r["tz"]),
                coldry=coldry, wkl=[w for row in wkl7 for w in row], altz=list(r["altz"]))
