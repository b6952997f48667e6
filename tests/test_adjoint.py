"""Tangent-linear and adjoint of the FP64 solve (rrtmg_sw_tl_c / rrtmg_sw_ad_c).

The objective J (TOA upward flux, surface net flux, sum of heating rates,
weighted) of the smooth model is checked three ways on McICA-cloudy columns
with frozen subcolumn masks:
  - the tangent-linear dJ along a random direction against FP64 central
    differences of J with relative step 1e-6 (tolerance 1e-6 relative to the
    largest |dJ|).  The heating-rate sum weighs net fluxes by heatfac/dp,
    ~3e3 for the 0.003 hPa top layers of a 0.01 hPa model top, where the
    FP64 rounding of J alone would exceed 1e-6 of a 1e-6 difference
    quotient; objectives with that sum are checked on columns topped at
    5 hPa (thinnest layer ~1 hPa);
  - the adjoint gradient dotted with the same direction against the
    tangent-linear dJ (tolerance 1e-9 relative);
  - the adjoint with stored and with recomputed local Jacobians against each
    other (tolerance 1e-12 relative).
"""
import numpy as np
import pytest

from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

pytestmark = pytest.mark.gpu

WEIGHTS = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (0.5, -1.0, 2.0)]


@pytest.fixture(scope="module")
def gpu():
    from rrtmg_sw_gb300 import build, interface
    build.build()
    interface.rrtmg_sw_ini(1.004e3)
    interface.set_form(interface.FORM_FP64)
    return interface


def case(ncol=8, nlay=30, seed=61, clouds=True, ptop=0.01):
    c = make_columns(ncol, nlay, seed, clouds=clouds, ptop=ptop)
    kw = gcm_inputs(c, icld=2 if clouds else 0, iaer=0)
    cl = None
    if clouds:
        cl = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
                  rel=c["rel"])
    return kw, cl


def direction(kw, cl, seed):
    """Relative perturbations of every differentiated input."""
    rng = np.random.default_rng(seed)
    d = {}
    for k in ("tlay", "h2ovmr", "o3vmr"):
        d[k] = rng.uniform(-1.0, 1.0, kw[k].shape) * kw[k]
    for k in ("clwp", "ciwp"):
        d[k] = rng.uniform(-1.0, 1.0, kw["tlay"].shape) * (cl[k] if cl is not None else 0.0)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        d[k] = rng.uniform(-1.0, 1.0, kw[k].shape) * kw[k]
    return d


def shifted(kw, cl, d, h):
    kw2 = dict(kw)
    for k in ("tlay", "h2ovmr", "o3vmr", "asdir", "asdif", "aldir", "aldif"):
        kw2[k] = kw[k] + h * d[k]
    cl2 = None
    if cl is not None:
        cl2 = dict(cl)
        for k in ("clwp", "ciwp"):
            cl2[k] = cl[k] + h * d[k]
    return kw2, cl2


@pytest.mark.parametrize("weights", WEIGHTS)
def test_tangent_linear_matches_central_differences(gpu, weights):
    kw, cl = case(ptop=5.0 if weights[2] != 0.0 else 0.01)
    d = direction(kw, cl, 7)
    tl = gpu.rrtmg_sw_tl(kw, d, cl, weights)
    h = 1.e-6

    def J(step):
        k2, c2 = shifted(kw, cl, d, step)
        return gpu.rrtmg_sw_tl(k2, {}, c2, weights)["J"]

    fd = (J(h) - J(-h)) / (2.0 * h)
    scale = max(np.max(np.abs(fd)), 1e-300)
    err = np.max(np.abs(tl["dJ"] - fd)) / scale
    assert err <= 1e-6, (err, tl["dJ"], fd)


@pytest.mark.parametrize("weights", WEIGHTS)
def test_adjoint_is_transpose_of_tangent_linear(gpu, weights):
    kw, cl = case(seed=62)
    d = direction(kw, cl, 8)
    tl = gpu.rrtmg_sw_tl(kw, d, cl, weights)
    ad = gpu.rrtmg_sw_ad(kw, cl, weights)
    dot = np.zeros(kw["ncol"])
    for k in gpu.AD_LAYER:
        dot += np.sum(ad[k] * d[k], axis=1)
    for k in gpu.AD_SFC:
        dot += ad[k] * d[k]
    scale = max(np.max(np.abs(tl["dJ"])), 1e-300)
    assert np.max(np.abs(dot - tl["dJ"])) / scale <= 1e-9
    # the weighted objective can cancel (J ~ 0.2 from terms of ~400 W m-2): compare on the terms' scale
    np.testing.assert_allclose(ad["J"], tl["J"], rtol=1e-13, atol=1e-13 * np.max(np.abs(tl["J"])))


def test_stored_and_recomputed_jacobians_agree(gpu):
    kw, cl = case(seed=63)
    a = gpu.rrtmg_sw_ad(kw, cl, (0.5, -1.0, 2.0), store=True)
    b = gpu.rrtmg_sw_ad(kw, cl, (0.5, -1.0, 2.0), store=False)
    for k in ("J",) + gpu.AD_LAYER + gpu.AD_SFC:
        scale = max(np.max(np.abs(a[k])), 1e-300)
        assert np.max(np.abs(a[k] - b[k])) / scale <= 1e-12, k


def test_checkpointing_chosen_by_memory(gpu):
    # store = "auto" (-1 in the C ABI): the stored Jacobians' scratch of a small
    # case fits, so they are stored, and the result is that of store=True
    kw, cl = case(seed=65)
    a = gpu.rrtmg_sw_ad(kw, cl, (0.5, -1.0, 2.0), store="auto")
    assert gpu.lib().rrtmg_sw_last_ad_store_c() == 1
    b = gpu.rrtmg_sw_ad(kw, cl, (0.5, -1.0, 2.0), store=True)
    for k in ("J",) + gpu.AD_LAYER + gpu.AD_SFC:
        scale = max(np.max(np.abs(b[k])), 1e-300)
        assert np.max(np.abs(a[k] - b[k])) / scale <= 1e-12, k


def test_smooth_model_is_close_to_the_table_model(gpu):
    kw, cl = case(seed=64, clouds=False)
    ad = gpu.rrtmg_sw_ad(kw, cl, (1.0, 0.0, 0.0))
    res = gpu.rrtmg_sw(**kw, extra=True)
    np.testing.assert_allclose(ad["J"], res["swuflx"][:, -1], atol=0.5)


def config4_subset(ncol=256):
    """The first `ncol` columns of the 65 536-column x 60-layer McICA set the
    adjoint is timed on (icld=2, seed 20261203 + 4, model top 0.01 hPa)."""
    c = make_columns(65536, 60, 20261203 + 4, clouds=True)
    c = {k: (v[:ncol] if isinstance(v, np.ndarray) and v.shape[:1] == (65536,) else v) for k, v in c.items()}
    kw = gcm_inputs(c, icld=2, iaer=0)
    cl = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
              rel=c["rel"])
    return kw, cl


@pytest.mark.parametrize("weights", [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0)])
def test_config4_subset_tangent_linear_matches_central_differences(gpu, weights):
    # 256 columns x 60 layers: FD with relative step 1e-6 within 1e-6 of the
    # largest |dJ|.  The model is piecewise smooth: setcoef's table indices
    # (jt, jt1, indself, indfor) jump where a layer temperature crosses a
    # grid line, so a column where some layer's step crosses one has a kink
    # inside [-2h, 2h] and no central difference to compare with; those
    # columns are found by their central quotients at steps h and 2h
    # disagreeing (smooth columns agree to O(h^2), far below the threshold)
    # and are left out (about one per 256 columns).  The heating-rate sum is left to the
    # transpose check below: with this set's 0.01 hPa top its FD quotient is
    # dominated by the FP64 rounding of J (see the module docstring).
    kw, cl = config4_subset()
    d = direction(kw, cl, 17)
    tl = gpu.rrtmg_sw_tl(kw, d, cl, weights)
    h = 1.e-6

    def J(step):
        k2, c2 = shifted(kw, cl, d, step)
        return gpu.rrtmg_sw_tl(k2, {}, c2, weights)["J"]

    fd = (J(h) - J(-h)) / (2.0 * h)
    fd2 = (J(2.0 * h) - J(-2.0 * h)) / (4.0 * h)
    scale = max(np.max(np.abs(fd)), 1e-300)
    kink = np.abs(fd - fd2) > 5e-7 * scale
    assert kink.sum() <= 0.02 * kw["ncol"], int(kink.sum())
    err = np.max(np.abs(tl["dJ"] - fd)[~kink]) / scale
    assert err <= 1e-6, (err, int(kink.sum()))


def test_config4_subset_adjoint_is_transpose_of_tangent_linear(gpu):
    kw, cl = config4_subset()
    weights = (0.5, -1.0, 2.0)
    d = direction(kw, cl, 18)
    tl = gpu.rrtmg_sw_tl(kw, d, cl, weights)
    for store in (True, False):
        ad = gpu.rrtmg_sw_ad(kw, cl, weights, store=store)
        dot = np.zeros(kw["ncol"])
        for k in gpu.AD_LAYER:
            dot += np.sum(ad[k] * d[k], axis=1)
        for k in gpu.AD_SFC:
            dot += ad[k] * d[k]
        scale = max(np.max(np.abs(tl["dJ"])), 1e-300)
        assert np.max(np.abs(dot - tl["dJ"])) / scale <= 1e-9, store
