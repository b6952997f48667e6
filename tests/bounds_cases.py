"""Cases run by tests/test_bounds_check.py under a chosen build of the
library (RRTMG_SW_LIB): every entry point and option that reads the
coefficient tables.  Writes the FP64-form outputs to an .npz file; any
nonzero status (RRTMG_SW_EBOUNDS in a bounds-check build) raises."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def run():
    from rrtmg_sw_gb300 import interface as gi
    from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns
    gi.rrtmg_sw_ini(1.004e3)
    out = {}
    for form, tag in ((gi.FORM_FP64, "f64"), (gi.FORM_FP32, "f32")):
        gi.set_form(form)
        c = make_columns(40, 60, 501, clouds=True, aerosol=True, lat=True, night_frac=0.2)
        ncol, nlay = c["play"].shape
        alpha = gi.get_alpha(1, ncol, nlay, 5, 1, 0.0, c["dz"], c["lat"], 94, c["cldfrac"])
        cases = {
            "clear": (gcm_inputs(c, icld=0, iaer=0), None),
            "aer10_kiss2": (gcm_inputs(c, icld=2, iaer=10),
                            dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"],
                                 rei=c["rei"], rel=c["rel"])),
            "kiss5": (gcm_inputs(c, icld=5, iaer=0),
                      dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"],
                           rei=c["rei"], rel=c["rel"], alpha=alpha)),
            "mt2": (gcm_inputs(c, icld=2, iaer=0),
                    dict(permuteseed=224, irng=1, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"],
                         rei=c["rei"], rel=c["rel"])),
        }
        for name, (kw, cl) in cases.items():
            r = gi.rrtmg_sw(**kw, clouds=cl, extra=True, bands=True, idelm=0 if name == "clear" else 1)
            for k, v in r.items():
                out["%s_%s_%s" % (tag, name, k)] = v
        kw = gcm_inputs(c, icld=0, iaer=6)
        kw["ecaer"] = np.full((ncol, nlay, 6), 0.01)
        r = gi.rrtmg_sw(**kw, extra=True)
        out["%s_aer6_swuflx" % tag] = r["swuflx"]
        # non-McICA overcast layers with band optics (inflgsw = 0)
        cf = (c["cldfrac"] > 0.5).astype(float)
        kw = gcm_inputs(c, icld=2, iaer=0)
        kw["inflgsw"] = 0
        rng = np.random.default_rng(9)
        nm = dict(cldfrac=cf, ciwp=c["ciwp"] * cf, clwp=c["clwp"] * cf, rei=c["rei"], rel=c["rel"],
                  tauc=rng.uniform(0, 5, (14, ncol, nlay)) * cf[None], ssac=rng.uniform(0.8, 0.999, (14, ncol, nlay)),
                  asmc=rng.uniform(0.6, 0.9, (14, ncol, nlay)))
        nm["fsfc"] = nm["asmc"] ** 2
        r = gi.rrtmg_sw(**kw, clouds=nm, nomcica=True, extra=True)
        out["%s_nomcica_swdflx" % tag] = r["swdflx"]
    gi.set_form(gi.FORM_FP64)
    kw = gcm_inputs(c, icld=2, iaer=0)
    cl = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
              rel=c["rel"])
    ad = gi.rrtmg_sw_ad(kw, cl, (1.0, 1.0, 1.0))
    out["ad_J"] = ad["J"]
    out["ad_tlay"] = ad["tlay"]
    return out


if __name__ == "__main__":
    np.savez(sys.argv[1], **run())
