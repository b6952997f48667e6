"""Pin the oracle on the five iatm = 1 example runs (solar variability).

These runs (run_examples_std_atm/input_rrtm_MLS-clr-sza45-isolvar*) give a
user profile of 48 levels and 48 layer boundaries in pressure; the column
driver turns them into 47 layers with the profile builder rrtatm.f
(rrtmg_sw.1col.f90:1728-1768).  The oracle's restatement of that builder
(oracle/rrtatm.py) makes the layers from the records in
tests/golden/std_atm_iatm1_cases.json, the column driver's solar settings
come from orc_solar_factors, and the oracle's column mode must reproduce
every printed block of the reference's outputs (broadband and the 14 bands,
iout = 98) to print precision, as the iatm = 0 runs do
(test_oracle_golden.py).  A planted error of 1e-6 in the layer amounts
must break that agreement.

Properties of the builder itself: boundaries given as altitudes or as the
same levels' pressures give the same layers; an extra boundary inside a
layer, given as an altitude or as a pressure between levels, splits its
molecular amounts (exponential in altitude) without changing their sum;
the hydrostatic altitudes (CMPALT) of the run's pressures stay near its
given altitudes, and a profile on pressure levels equals the same profile
on those altitudes; the run's profile is the built-in mid-latitude summer
atmosphere, so unit codes taking its values give the same layers, and the
built-in atmosphere itself (MODEL = 2) the same pressures and temperatures;
the inputs outside the restated part raise.
"""
import copy
import json
import os

import numpy as np
import pytest

import pyoracle
import rrtatm

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "std_atm_iatm1_cases.json")))["cases"]
TOL = {"uflx": 5e-5, "difdflx": 5e-5, "dirdflx": 5e-5, "dflx": 5e-5, "fnet": 5e-7, "htr": 5e-6}


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    pyoracle.init(1.004e3)


def column_case(case, lay):
    """The column driver's inputs for one iatm = 1 run (rrtmg_sw.1col.f90:1391-1436, 1646-1660)."""
    iso, sv = case["isolvar"], case["solvar"]
    kw = {}
    if iso in (1, 2):
        kw["indsolvar"] = sv[:2]
    if iso == 1:
        kw["solcycfrac"] = case["solcycfrac"]
    if iso in (-1, 3):
        kw["bndsolvar"] = sv
    sf = pyoracle.solar_factors(iso, case["scon"], 1.0, case["juldat"], **kw)
    nl = lay["nlay"]
    z = [0.0] * nl
    return dict(nlay=nl, icld=case["icld"], iaer=case["iaer"], idelm=case["idelm"], imca=case["imca"], idcor=0,
                juldat=case["juldat"], inflag=0, iceflag=0, liqflag=0, isolvar=iso, zenith=case["zenith"],
                decorr_con=0.0, lat=0.0, svar=tuple(sf["svar"]), svar_bnd=sf["svar_bnd"], adjflux=sf["adjflux"],
                albedo=case["albedo"], pavel=lay["pavel"], tavel=lay["tavel"], pz=lay["pz"], tz=lay["tz"],
                coldry=lay["coldry"], wkl=lay["wkl"], dz=z, cldfrac=z, ciwp=z, clwp=z, rei=z, rel=z)


def misses(case, lay):
    """Printed values the oracle misses by more than print precision."""
    cc = column_case(case, lay)
    bad = []
    for b in case["expected"]:
        out = pyoracle.column_mode(cc, b["istart"], b["iend"])
        for k, tol in TOL.items():
            err = np.abs(out[k] - np.array(b[k]))
            bad += [(b["istart"], b["iend"], k, int(i), float(err[i])) for i in np.nonzero(err > tol + 1e-9)[0]]
    return bad


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_golden_blocks(case):
    assert case["icld"] == 0 and case["iaer"] == 0 and len(case["expected"]) == 15
    lay = rrtatm.readprof_layers(case["atm"])
    assert lay["nlay"] == 47
    # the level pressures are the printed pressure column (to its 4 significant digits)
    np.testing.assert_allclose(lay["pz"], case["expected"][0]["p"], rtol=2e-3)
    bad = misses(case, lay)
    assert not bad, bad[:10]


def test_planted_layer_error_is_caught():
    case = CASES[0]
    lay = rrtatm.readprof_layers(case["atm"])
    lay["wkl"] = [w * (1.0 + 1e-6) for w in lay["wkl"]]
    assert len(misses(case, lay)) > 10


def altitude_records(atm, extra=()):
    """The same run with its boundaries given as the levels' altitudes (IBMAX > 0)."""
    a = copy.deepcopy(atm)
    z = sorted([lv["z"] for lv in a["levels"]] + list(extra))
    a["ibmax_b"] = len(z)
    a["bnd"] = z
    a["h1"], a["h2"] = z[0], z[-1]
    return a


def test_pressure_and_altitude_boundaries_agree():
    atm = CASES[0]["atm"]
    p = rrtatm.readprof_layers(atm)
    z = rrtatm.readprof_layers(altitude_records(atm))
    for k in ("pavel", "tavel", "pz", "tz", "coldry", "wkl"):
        assert p[k] == z[k], k


def test_split_layer_keeps_molecular_amounts():
    atm = CASES[0]["atm"]
    whole = rrtatm.atmpth(altitude_records(atm))
    # 25.0-27.5 km is layer 26; a boundary at 26.1 km splits it in two path layers
    split = rrtatm.atmpth(altitude_records(atm, extra=(26.1,)))
    assert split["nlayrs"] == whole["nlayrs"] + 1
    l = [i for i in range(1, whole["nlayrs"] + 1) if whole["altz"][i - 1] == 25.0][0]
    for k in range(7):
        a, s = whole["amount"][k], split["amount"][k]
        assert s[l] + s[l + 1] == pytest.approx(a[l], rel=1e-12)
        assert s[:l] == a[:l]
        assert s[l + 2:] == a[l + 1:]
    assert split["pz"][l] < split["pz"][l - 1] and split["pz"][l] > split["pz"][l + 1]


def test_cmpalt_heights_of_the_example_profile():
    # the run's profile gives both altitudes and pressures: the hydrostatic
    # altitudes of its pressures stay within 0.5 % of the given ones
    atm = CASES[0]["atm"]
    z, p, t, den = rrtatm.nsmdl(atm["levels"], 7, 0.0, 48, 45.0, 6371.23)
    zc = rrtatm.cmpalt(p, t, [d[0] for d in den], z[0], 45.0, 6371.23)
    assert zc[0] == z[0]
    assert all(abs(a - b) <= 0.005 * b + 0.01 for a, b in zip(zc, z))
    assert all(zc[i] > zc[i - 1] for i in range(1, len(zc)))


def test_pressure_level_profile_takes_cmpalt_heights():
    atm = CASES[0]["atm"]
    onp = copy.deepcopy(atm)
    onp["immax_b"] = -atm["immax_b"]
    z, p, t, den = rrtatm.nsmdl(atm["levels"], 7, 0.0, 48, 45.0, 6371.23)
    zc = rrtatm.cmpalt(p, t, [d[0] for d in den], z[0], 45.0, 6371.23)
    onz = copy.deepcopy(atm)
    for lv, h in zip(onz["levels"], zc):
        lv["z"] = h
    a, b = rrtatm.readprof_layers(onp), rrtatm.readprof_layers(onz)
    for k in ("pavel", "tavel", "pz", "tz", "coldry", "wkl", "altz"):
        assert a[k] == b[k], k


def test_boundary_between_pressure_levels():
    atm = CASES[0]["atm"]
    split = copy.deepcopy(atm)
    i = split["bnd"].index(19.07)
    split["bnd"].insert(i, 23.0)
    split["ibmax_b"] = -(abs(atm["ibmax_b"]) + 1)
    whole, part = rrtatm.atmpth(atm), rrtatm.atmpth(split)
    assert part["nlayrs"] == whole["nlayrs"] + 1
    l = [k for k in range(1, whole["nlayrs"] + 1) if whole["pz"][k - 1] == 27.7][0]
    assert part["pz"][l] == pytest.approx(23.0, rel=5e-3)
    assert part["pz"][l - 1] == 27.7 and part["pz"][l + 1] == 19.07
    for k in range(7):
        assert part["amount"][k][l] + part["amount"][k][l + 1] == pytest.approx(whole["amount"][k][l], rel=1e-12)


def test_unit_codes_take_the_model_atmosphere():
    # the run's profile is the mid-latitude summer atmosphere (model 2) at its
    # 48 lowest levels: unit code 2 for the temperatures and all seven species
    # (DEFALT at the model's own altitudes) must give the same layers
    atm = CASES[0]["atm"]
    coded = copy.deepcopy(atm)
    for lv in coded["levels"]:
        lv["jchart"] = "2"
        lv["jchar"] = "2222222"
        lv["t"], lv["wmol"] = 0.0, [0.0] * 7
    a, b = rrtatm.readprof_layers(atm), rrtatm.readprof_layers(coded)
    for k in a:
        assert a[k] == b[k], k


def test_model_atmosphere_interpolation_between_levels():
    # 4-point Lagrange interpolation in altitude: a cubic through the four
    # neighbouring levels of the model's table
    d = rrtatm.afgl()
    z = 2.6
    p, t, junit, wmol = rrtatm.defalt(z, 0.0, 0.0, 2, 2, [2] * 7, [0.0] * 7, 7)
    i = [1, 2, 3, 4]
    for got, tab, log in [(t, d["t"][1], False), (p, d["p"][1], True)] + \
            [(wmol[k], d["amol"][1][k], False) for k in range(7)]:
        y = np.log([tab[j] for j in i]) if log else [tab[j] for j in i]
        ref = np.polyval(np.polyfit([d["alt"][j] for j in i], y, 3), z)
        assert (np.log(got) if log else got) == pytest.approx(ref, rel=1e-9, abs=1e-12)
    assert junit == [10] * 7


def test_unit_codes_on_pressure_levels():
    # DEFALT_P at the model's own pressures returns its table values: a
    # profile on pressure levels with unit code 2 equals the same profile
    # with the values written out
    atm = copy.deepcopy(CASES[0]["atm"])
    atm["immax_b"] = -atm["immax_b"]
    coded = copy.deepcopy(atm)
    for lv in coded["levels"]:
        lv["jchart"] = "2"
        lv["jchar"] = "2222222"
        lv["t"], lv["wmol"] = 0.0, [0.0] * 7
    a, b = rrtatm.readprof_layers(atm), rrtatm.readprof_layers(coded)
    for k in a:
        assert a[k] == b[k], k
    # between the model's pressures: a cubic in ln p through the four neighbours
    d = rrtatm.afgl()
    p = 700.0
    t, junit, wmol = rrtatm.defalt_p(p, 0.0, 2, [2] * 7, [0.0] * 7, 7)
    i = [2, 3, 4, 5]
    x = np.log([d["p"][1][j] for j in i])
    for got, tab in [(t, d["t"][1])] + [(wmol[k], d["amol"][1][k]) for k in range(7)]:
        ref = np.polyval(np.polyfit(x, [tab[j] for j in i], 3), np.log(p))
        assert got == pytest.approx(ref, rel=1e-9, abs=1e-12)
    assert junit == [10] * 7


def test_builtin_model_atmosphere():
    # MODEL = 2 takes the same levels from the built-in table but densities
    # from its tabulated air density (MDLATM) rather than the ideal gas
    # (CONVRT): pressures and temperatures agree exactly, amounts to 1e-3,
    # and the printed tables to a few hundredths
    case = CASES[0]
    atm = copy.deepcopy(case["atm"])
    atm["model"] = 2
    a, b = rrtatm.readprof_layers(case["atm"]), rrtatm.readprof_layers(atm)
    for k in ("pavel", "tavel", "pz", "tz"):
        assert a[k] == b[k], k
    np.testing.assert_allclose(b["wkl"], a["wkl"], rtol=1e-3)
    cc = column_case(case, b)
    for blk in case["expected"]:
        out = pyoracle.column_mode(cc, blk["istart"], blk["iend"])
        for k in ("uflx", "dflx", "dirdflx", "difdflx", "fnet", "htr"):
            assert np.max(np.abs(out[k] - np.array(blk[k]))) <= 0.05, (blk["istart"], k)


@pytest.mark.parametrize("change", ["trace_species", "slant", "autolayer"])
def test_unrestated_inputs_raise(change):
    atm = copy.deepcopy(CASES[0]["atm"])
    if change == "trace_species":
        atm["model"] = 2
        atm["nmol"] = 8
    elif change == "slant":
        atm["range"] = 10.0
    else:
        atm["ibmax_b"] = 0
    with pytest.raises(NotImplementedError):
        rrtatm.atmpth(atm)
