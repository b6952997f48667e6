"""Benchmark: sunlit columns/s of the fused McICA shortwave solve on one GB300.

Workload (N=1): 262,144 columns x 60 layers, McICA clouds with
exponential-random overlap (icld=5, idcor=1, KISS subcolumns generated in
the kernel), inflgsw=2/iceflgsw=3/liqflgsw=1, no aerosol, all columns
sunlit.  A step is one call of the fused entry point over the whole batch.

value            FP32-form sunlit columns/s, kernel only, inputs resident in
                 HBM (~1.6 GB, larger than L2, so no flush is needed)
e2e              the same through the host-array C-ABI entry point
                 (rrtmg_sw_mcica_c): H2D of the inputs from pinned memory,
                 the solve, D2H of the six output arrays, every step
fp64             the plain FP64 form on the same inputs (the metric's
                 comparison), and the FP32 form's largest errors against it
fp32_counters    cells the FP32 form redid in FP64, and its fallbacks
headline_iaer10  the same workload with iaer=10 aerosols, both forms
clear_1024x60, mcica_aer_16384x60
                 the 1024-column clear-sky and 16384-column McICA + aerosol
                 configurations: CPU oracle, GPU FP64 and FP32 columns/s,
                 errors against the oracle
batch            48 ragged instances in one persistent launch (FP64 form)
cpu_baseline     the FP64 oracle (oracle/, all host threads) over the whole
                 headline workload
fp32_vs_oracle   the FP32 form against that oracle (max and RMS per field);
                 per-level max / RMS go to stderr as one JSON line
fp64_vs_oracle   the FP64 form against it, with the fraction of elements
                 within |d| <= 1e-9 |ref| + floor

``--quick`` keeps the headline only (oracle on a bounded sample).
``--impl reference`` times the FP64 CPU restatement of the reference
(oracle/, all host threads) on a bounded sample of the same workload.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NCOL, NLAY = 262144, 60
SEED = 20261203 + 3
METRIC = "sunlit columns/s, FP32 form vs plain FP64, same GB300, <=0.05 W/m2 flux err"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300")
    p.add_argument("--ncol", type=int, default=NCOL)
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--quick", action="store_true",
                   help="headline only: no iaer=10 / small-config / batch legs, oracle on a bounded sample")
    p.add_argument("--workload", default="fp32", choices=["fp32", "batch", "adjoint"],
                   help="fp32: the FP32-form headline; batch: 48 ragged instances in one launch (FP64 form)")
    p.add_argument("--instances", type=int, default=48)
    p.add_argument("--batch-form", default="fp64", choices=["fp64", "fp32"],
                   help="arithmetic form of --workload batch (the batching configuration names FP64)")
    p.add_argument("--irng", type=int, default=0, choices=[0, 1],
                   help="McICA generator of the fused solve: 0 KISS, 1 MT19937 (one stream per call, GCM order)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def inputs(ncol, seed):
    from rrtmg_sw_gb300.synthetic import make_columns
    c = make_columns(ncol, NLAY, seed, clouds=True, lat=True)
    return c


def algorithmic_flops_per_column(nlay, cloudy_cells_per_col):
    # itemised from the reference's statements: per (g, layer) 257, per (g, level) 48,
    # per cloudy (g, layer) 171 (cloud reftra + cldprmc)
    return 112 * (257 * nlay + 48 * (nlay + 1)) + 171 * cloudy_cells_per_col


# DRAM bytes per column of the FP32 form's kernels measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) in captures at 32768 columns x
# 60 layers, McICA icld=5; the traffic is per column pair, so a launch's
# traffic scales with its columns.
PROFILED_DRAM_BYTES_PER_COLUMN = {"fp32 scratch": 28.38e9 / 32768,
                                  "fp32 tiled": (331.934208e6 + 114.524672e6) / 32768}
# the tiled kernel's preparation kernel (k_tiled_prep), same capture
PROFILED_PREP_DRAM_BYTES_PER_COLUMN = (222.937088e6 + 209.511936e6) / 32768


def algorithmic_bytes_per_column(nlay):
    # FP64 interface, fused McICA: 7 gas/state layer arrays + plev + 4 albedos + coszen,
    # physical clouds 5L + alpha L, outputs 4 (L+1) + 2 L
    return 8 * (7 * nlay + (nlay + 1) + 5 + 6 * nlay + 4 * (nlay + 1) + 2 * nlay)


class Clocks:
    """nvidia-smi sampler for the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def run_reference(args):
    """Time the FP64 CPU restatement (oracle) on a bounded sample."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from rrtmg_sw_gb300.synthetic import gcm_inputs
    cores = os.cpu_count() or 1
    sample = int(os.environ.get("RRTMG_REF_SAMPLE", "0")) or max(64, 48 * cores)
    c = inputs(sample, SEED)
    alpha = pyoracle.get_alpha(sample, NLAY, 5, 1, 0.0, c["dz"].ravel(order="F"), c["lat"], 94,
                               c["cldfrac"].ravel(order="F"))
    z14 = np.zeros(14 * sample * NLAY)

    def step():
        m = pyoracle.mcica_subcol_sw(sample, NLAY, 5, 112, 0, *(c[k].ravel(order="F") for k in
                                                                ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                     z14, z14 + 1.0, z14, z14, alpha)
        names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
        kw = gcm_inputs(c, icld=5, iaer=0, mcica=tuple(m[k] for k in names))
        inp = {k: kw[k] for k in pyoracle.GCM_INPUTS + pyoracle.MCICA_INPUTS + pyoracle.AER_INPUTS}
        pyoracle.rrtmg_sw(sample, NLAY, 5, 0, inp, nthreads=cores)

    for _ in range(max(args.warmup, 1)):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    v = sample / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "columns/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "262144x60 McICA icld=5 idcor=1 (bounded sample of %d columns per step)" % sample,
                   "ncol": NCOL, "nlay": NLAY},
        "cpu_baseline": {"value": v, "unit": "columns/s", "cores": cores, "kind": "port",
                         "sample": "%d columns x %d layers per step, McICA + solve, OpenMP over columns" % (sample, NLAY)},
        "e2e": {"value": v, "unit": "columns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_batch(args):
    """The ragged-batch configuration alone (see batch_workload), one JSON line."""
    import torch
    from rrtmg_sw_gb300 import build, interface as gi
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    dev = torch.device("cuda", 0)
    r = batch_workload(args, gi, torch, dev)
    steps = max(1, args.steps // 5)
    line = {"metric": "sunlit columns/s, %d ragged instances in one persistent launch (%s form)" %
                      (r["instances"], r["form"].upper()),
            "value": r["value"], "unit": "columns/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if r["form"] == "fp32" else "f64", "data": "synthetic",
            "config": {"workload": "%d instances, ncol log-uniform 512..131072, nlay in {40,47,60,72,91,137}, 40%% "
                                   "night, McICA icld=2, %s form" % (r["instances"], r["form"].upper()),
                       "columns": r["columns"], "sunlit": r["sunlit"]},
            "sum_of_single_calls_ms": r["sum_of_single_calls_ms"], "autotuner": r["autotuner"],
            "instances": r["per_instance"]}
    print(json.dumps(line))


def adjoint_workload(args, gi, k=3, recompute=True):
    """Adjoint cost: 65536 columns x 60 layers, McICA clouds (icld=2, masks
    frozen), objective TOA up + surface net + heating-rate sum; forward,
    tangent-linear and adjoint (stored / recomputed local Jacobians) through
    the host-array C ABI, each timed end to end (best of k after one
    untimed call)."""
    from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns
    gi.set_form(gi.FORM_FP64)
    ncol = args.ncol if args.ncol != NCOL else 65536
    c = make_columns(ncol, NLAY, 20261203 + 4, clouds=True)
    kw = gcm_inputs(c, icld=2, iaer=0)
    for key in MC_NAMES:
        kw[key] = None  # fused McICA: the subcolumn arrays are not passed
    cl = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
              rel=c["rel"])
    w = (1.0, 1.0, 1.0)

    def best(f):
        f()
        ts = []
        for _ in range(k):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        return min(ts) * 1e3

    fwd = best(lambda: gi.rrtmg_sw(**kw, clouds=cl))
    gi.set_form(gi.FORM_FP32)
    fwd32 = best(lambda: gi.rrtmg_sw(**kw, clouds=cl))
    gi.set_form(gi.FORM_FP64)
    d = {key: np.ones_like(kw["tlay"]) for key in gi.AD_LAYER}
    tl = best(lambda: gi.rrtmg_sw_tl(kw, d, cl, w))
    ad_s = best(lambda: gi.rrtmg_sw_ad(kw, cl, w, store=True))
    res = {"workload": "%d columns x %d layers, McICA icld=2, objective TOA up + sfc net + HR sum, host-array calls "
                       "end to end, best of %d" % (ncol, NLAY, k),
           "forward_fp64_ms": fwd, "forward_fp32_ms": fwd32, "tangent_linear_ms": tl, "adjoint_store_ms": ad_s,
           "adjoint_store_vs_fp64_forward": ad_s / fwd, "adjoint_store_vs_fp32_forward": ad_s / fwd32}
    if recompute:
        ad_r = best(lambda: gi.rrtmg_sw_ad(kw, cl, w, store=False))
        res.update(adjoint_recompute_ms=ad_r, adjoint_recompute_vs_fp64_forward=ad_r / fwd)
    return res


def run_adjoint(args):
    """The adjoint configuration alone (see adjoint_workload), one JSON line."""
    from rrtmg_sw_gb300 import build, interface as gi
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    r = adjoint_workload(args, gi)
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    # per-CTA scratch (doubles) of the adjoint kernel, 3 resident CTAs per SM
    slot = lambda fields: ((NLAY + 1) * fields * 224 + 2 * 15 * NLAY * 4) * 8 * 3
    line = {"metric": "adjoint cost relative to the FP64 forward it differentiates (host-array calls, end to end)",
            "value": r["adjoint_store_vs_fp64_forward"], "unit": "x forward", "n_gpus": 1,
            "higher_is_better": False, "config": {"workload": r["workload"]},
            "scratch_bytes_store": slot(45) * sms, "scratch_bytes_recompute": slot(20) * sms}
    line.update({k: v for k, v in r.items() if k != "workload"})
    print(json.dumps(line))


FIELDS = ("swuflx", "swdflx", "swuflxc", "swdflxc", "swhr", "swhrc")
HRF = ("swhr", "swhrc")
MC_NAMES = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")


class DevCase:
    """One rrtmg_sw call's arrays in HBM and its C-ABI structs (device
    pointers): clear sky, or McICA generated inside the solve (icld >= 1)."""

    def __init__(self, gi, torch, dev, c, icld, iaer, alpha=None, irng=0):
        self.gi, self.torch = gi, torch
        self.ncol, self.nlay = c["play"].shape
        T = lambda x: torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).to(dev)
        ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), gi._dp)
        names = ["play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif", "aldir",
                 "aldif", "coszen"]
        if iaer == 10:
            names += ["tauaer", "ssaaer", "asmaer"]
        self.d = {k: T(c[k]) for k in names}
        n, L = self.ncol, self.nlay
        self.o = {k: torch.empty(n * (L if k in HRF else L + 1), dtype=torch.float64, device=dev) for k in FIELDS}
        a = gi.RrtmgSwArgs()
        a.ncol, a.nlay, a.icld, a.iaer = n, L, icld, iaer
        for k, v in list(self.d.items()) + list(self.o.items()):
            setattr(a, k, ptr(v))
        a.adjes, a.dyofyr, a.scon, a.isolvar = 1.0, 0, 1360.85, 0
        a.inflgsw, a.iceflgsw, a.liqflgsw = 2, 3, 1
        a.idelm = 1
        self.a, self.cl = a, None
        if icld >= 1:
            cn = ["cldfrac", "ciwp", "clwp", "rei", "rel"]
            self.dc = {k: T(c[k]) for k in cn}
            if alpha is not None:
                self.dc["alpha"] = T(alpha)
            cl = gi.RrtmgSwClouds()
            cl.permuteseed, cl.irng = 112, irng
            for k, v in self.dc.items():
                setattr(cl, k, ptr(v))
            self.cl = cl
        self.input_bytes = sum(v.numel() * 8 for v in self.d.values()) + \
            (sum(v.numel() * 8 for v in self.dc.values()) if icld >= 1 else 0)

    def run(self, sid):
        self.gi.rrtmg_sw_dev(self.a, sid, self.cl)

    def outputs(self):
        n, L = self.ncol, self.nlay
        return {k: v.cpu().numpy().reshape((n, L if k in HRF else L + 1), order="F") for k, v in self.o.items()}


def time_steps(torch, stream, fn, steps, warmup, world=1):
    """Mean ms per step on `stream` by CUDA events, after warm-up, with a
    synchronize (and, on several ranks, a barrier) on both sides; max over ranks."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def oracle_solve(c, icld, iaer, alpha=None, irng=0, chunk=4096):
    """The FP64 oracle over all columns of c, in column chunks (KISS
    subcolumn streams are seeded per column, so chunks give the whole call's
    results); returns (outputs, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from rrtmg_sw_gb300.synthetic import gcm_inputs
    ncol, nlay = c["play"].shape
    cores = os.cpu_count() or 1
    out = {k: np.empty((ncol, nlay if k in HRF else nlay + 1)) for k in FIELDS}
    t0 = time.perf_counter()
    for j0 in range(0, ncol, chunk):
        j1 = min(ncol, j0 + chunk)
        n = j1 - j0
        cs = {k: (v[j0:j1] if isinstance(v, np.ndarray) and v.shape[:1] == (ncol,) else v) for k, v in c.items()}
        mc = None
        if icld:
            z14 = np.zeros(14 * n * nlay)
            al = np.zeros(n * nlay) if alpha is None else np.asfortranarray(alpha[j0:j1]).ravel(order="F")
            m = pyoracle.mcica_subcol_sw(n, nlay, icld, 112, irng, *(np.asfortranarray(cs[k]).ravel(order="F") for k
                                                                    in ("play", "cldfrac", "ciwp", "clwp", "rei",
                                                                        "rel")), z14, z14 + 1.0, z14, z14, al)
            mc = tuple(m[k] for k in MC_NAMES)
        kw = gcm_inputs(cs, icld=icld, iaer=iaer, mcica=mc)
        inp = {k: kw[k] for k in pyoracle.GCM_INPUTS + pyoracle.MCICA_INPUTS + pyoracle.AER_INPUTS}
        o = pyoracle.rrtmg_sw(n, nlay, icld, iaer, inp, nthreads=cores)
        for k in FIELDS:
            out[k][j0:j1] = o[k].reshape((n, out[k].shape[1]), order="F")
    return out, time.perf_counter() - t0


def g3(x):
    return float("%.3g" % x)


def diff_summary(got, ref):
    """Max |d| over fluxes (W/m2) and heating rates (K/day), each field's
    max / RMS, and the elementwise rule |d| <= 1e-9 |ref| + floor (1e-9 W/m2,
    1e-8 K/day) as the fraction of elements that meet it."""
    mx, rms, ok, tot = {}, {}, 0, 0
    for k in FIELDS:
        d = np.abs(got[k] - ref[k])
        mx[k] = g3(d.max())
        rms[k] = g3(np.sqrt(np.mean(d * d)))
        ok += int(np.sum(d <= 1e-9 * np.abs(ref[k]) + (1e-8 if k in HRF else 1e-9)))
        tot += d.size
    return {"max_dF": max(mx[k] for k in FIELDS if k not in HRF), "max_dHR": max(mx[k] for k in HRF),
            "max": mx, "rms": rms, "frac_within_1e-9_rel": g3(ok / tot)}


def per_level(got, ref):
    """Max and RMS over columns of |dF| per level (surface first, max over
    the four flux fields) and |dHR| per layer (max over both)."""
    fl = np.max([np.abs(got[k] - ref[k]) for k in FIELDS if k not in HRF], axis=0)
    fr = np.sqrt(np.max([np.mean((got[k] - ref[k]) ** 2, axis=0) for k in FIELDS if k not in HRF], axis=0))
    hl = np.max([np.abs(got[k] - ref[k]) for k in HRF], axis=0)
    hr = np.sqrt(np.max([np.mean((got[k] - ref[k]) ** 2, axis=0) for k in HRF], axis=0))
    f = lambda v: [float("%.2g" % x) for x in v]
    return {"dF_max": f(fl.max(axis=0)), "dF_rms": f(fr), "dHR_max": f(hl.max(axis=0)), "dHR_rms": f(hr)}


def small_workload(gi, torch, dev, sid, name, ncol, icld, iaer, seed):
    """One of the benchmark configurations at its own size (1024 x 60 clear,
    16384 x 60 McICA + aerosol): CPU oracle, GPU FP64 and FP32 forms
    (device-resident, CUDA events), both against the oracle."""
    from rrtmg_sw_gb300.synthetic import make_columns
    c = make_columns(ncol, NLAY, seed, clouds=icld > 0, aerosol=iaer == 10)
    dc = DevCase(gi, torch, dev, c, icld, iaer)
    sunlit = int((c["coszen"] > 0).sum())
    res = {"workload": name}
    for form, tag in ((gi.FORM_FP64, "fp64"), (gi.FORM_FP32, "fp32")):
        gi.set_form(form)
        ms = time_steps(torch, torch.cuda.current_stream(dev), lambda: dc.run(sid), 10, 3)
        res[tag] = {"value": sunlit / (ms / 1e3), "ms": g3(ms), "kernel": gi.last_kernel()}
    gi.set_form(gi.FORM_FP64)
    dc.run(sid)
    o64 = dc.outputs()
    gi.set_form(gi.FORM_FP32)
    dc.run(sid)
    o32 = dc.outputs()
    ref, dt = oracle_solve(c, icld, iaer)
    res["cpu_oracle"] = {"value": sunlit / dt, "cores": os.cpu_count() or 1}
    s64, s32 = diff_summary(o64, ref), diff_summary(o32, ref)
    res["fp64"].update(max_dF=s64["max_dF"], max_dHR=s64["max_dHR"], frac_within_1e_9_rel=s64["frac_within_1e-9_rel"])
    res["fp32"].update(max_dF=s32["max_dF"], max_dHR=s32["max_dHR"])
    del dc
    torch.cuda.empty_cache()
    return res


def batch_workload(args, gi, torch, dev, per_instance=True):
    """48 ragged instances (ncol log-uniform in 512..131072, nlay from
    {40,47,60,72,91,137}, 40 % night columns, McICA clouds icld=2 with
    inflgsw=2/iceflgsw=3/liqflgsw=1) in one persistent launch replayed from a
    CUDA graph; per-instance figures from single calls."""
    from rrtmg_sw_gb300.synthetic import make_columns
    fp32 = args.batch_form == "fp32"
    gi.set_form(gi.FORM_FP32 if fp32 else gi.FORM_FP64)
    rng = np.random.default_rng(20261203 + 2)
    insts = []
    for i in range(args.instances):
        ncol = int(round(np.exp(rng.uniform(np.log(512), np.log(131072)))))
        nlay = int(rng.choice([40, 47, 60, 72, 91, 137]))
        c = make_columns(ncol, nlay, 20261203 + 2 + 1000 * i, clouds=True, night_frac=0.4)
        dc = DevCase(gi, torch, dev, c, 2, 0)
        insts.append(dict(dc=dc, ncol=ncol, nlay=nlay, sunlit=int((c["coszen"] > 0).sum())))
    stream = torch.cuda.current_stream(dev)
    sid = stream.cuda_stream
    plan = gi.BatchPlan([x["dc"].a for x in insts], [x["dc"].cl for x in insts], stream=sid)
    ms = time_steps(torch, stream, lambda: plan.run(sid), max(1, args.steps // 5), max(1, args.warmup - 1))
    sunlit = sum(x["sunlit"] for x in insts)
    per = []
    for x in insts:  # each instance alone through rrtmg_sw_mcica_dev_c
        m1 = time_steps(torch, stream, lambda: x["dc"].run(sid), 1, 1)
        per.append({"ncol": x["ncol"], "nlay": x["nlay"], "sunlit": x["sunlit"], "single_ms": g3(m1),
                    "single_columns_per_s": g3(x["sunlit"] / (m1 / 1e3))})
    info = plan.info()
    plan.close()
    gi.set_form(gi.FORM_FP64)
    res = {"value": sunlit / (ms / 1e3), "unit": "sunlit columns/s", "ms_per_step": ms,
           "form": "fp32" if fp32 else "fp64", "instances": len(insts), "columns": sum(x["ncol"] for x in insts),
           "sunlit": sunlit, "sum_of_single_calls_ms": sum(p["single_ms"] for p in per),
           "autotuner": info}
    if per_instance:
        res["per_instance"] = per
    else:
        # compact: (ncol, nlay, sunlit columns/s of the instance called alone)
        res["per_instance_single"] = [[p["ncol"], p["nlay"], int(p["single_columns_per_s"])] for p in per]
    del insts
    torch.cuda.empty_cache()
    return res


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from rrtmg_sw_gb300 import build, interface as gi
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    ncol = args.ncol
    c = inputs(ncol, SEED + rank)
    # alpha for icld=5/idcor=1 on the device (get_alpha)
    alpha = gi.get_alpha(1, ncol, NLAY, 5, 1, 0.0, c["dz"], c["lat"], 94, c["cldfrac"])
    dev = torch.device("cuda", local)
    hc = DevCase(gi, torch, dev, c, 5, 0, alpha=alpha, irng=args.irng)
    stream = torch.cuda.current_stream(dev)
    sid = stream.cuda_stream

    import tempfile
    clk_path = os.path.join(tempfile.gettempdir(), "rrtmg_sw_bench_clocks_%d.csv" % os.getpid())
    # the dominant kernel's launches timed alone, on the launching stream
    gi.set_form(gi.FORM_FP32)
    with Clocks(clk_path) as clk:
        ms32 = time_steps(torch, stream, lambda: hc.run(sid), args.steps, args.warmup, world)
    clocks = clk.summary()
    kernel = {0: "fp64", 1: "fp32 scratch", 2: "fp32 tiled"}.get(gi.last_kernel(), "?")
    stats = gi.last_fp32_stats()
    launches_per_step = gi.last_launch_count()
    res32 = hc.outputs()
    sunlit = int((c["coszen"] > 0).sum())
    ms64 = None
    if not args.no_fp64:
        gi.set_form(gi.FORM_FP64)
        ms64 = time_steps(torch, stream, lambda: hc.run(sid), max(2, args.steps // 5), 1, world)
        res64 = hc.outputs()
        d64 = diff_summary(res32, res64)
    gi.set_form(gi.FORM_FP32)

    # irng = 1: the MT19937 generator alone on the call's stream (icld 5: two draws per cell)
    mt_stream = None
    if args.irng == 1:
        nmt = 2 * 112 * ncol * NLAY
        buf = torch.empty(nmt, dtype=torch.int32, device=dev)
        mt_ms = time_steps(torch, stream, lambda: gi.mt_stream_dev(112, nmt, buf.data_ptr(), 0, sid), 3, 1)
        mt_stream = {"words": nmt, "ms": mt_ms, "gwords_per_s": nmt / (mt_ms / 1e3) / 1e9,
                     "write_gbs": 4 * nmt / (mt_ms / 1e3) / 1e9}
        del buf

    # end to end through the host-array C ABI (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        pin = lambda x: torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).pin_memory()
        h = {k: pin(c[k]) for k in ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr",
                                    "n2ovmr", "o2vmr", "asdir", "asdif", "aldir", "aldif", "coszen", "cldfrac",
                                    "ciwp", "clwp", "rei", "rel")}
        h["alpha"] = pin(alpha)
        ho = {k: torch.empty(v.numel(), dtype=torch.float64).pin_memory() for k, v in hc.o.items()}
        ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), gi._dp)
        ah = gi.RrtmgSwArgs()
        ah.ncol, ah.nlay, ah.icld, ah.iaer = ncol, NLAY, 5, 0
        for k in ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
                  "asdir", "asdif", "aldir", "aldif", "coszen"):
            setattr(ah, k, ptr(h[k]))
        ah.adjes, ah.dyofyr, ah.scon, ah.isolvar = 1.0, 0, 1360.85, 0
        ah.inflgsw, ah.iceflgsw, ah.liqflgsw = 2, 3, 1
        for k, v in ho.items():
            setattr(ah, k, ptr(v))
        ah.idelm = 1
        ch = gi.RrtmgSwClouds()
        ch.permuteseed, ch.irng = 112, args.irng
        for k in ("cldfrac", "ciwp", "clwp", "rei", "rel", "alpha"):
            setattr(ch, k, ptr(h[k]))
        used = ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif", "aldir",
                "aldif", "coszen", "cldfrac", "ciwp", "clwp", "rei", "rel", "alpha")
        h2d = int(sum(h[k].numel() * 8 for k in used))
        d2h = int(sum(v.numel() * 8 for v in ho.values()))
        for _ in range(args.warmup):
            gi._check(gi.lib().rrtmg_sw_mcica_c(C.byref(ah), C.byref(ch)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_steps = max(3, args.steps // 2)
        for _ in range(e_steps):
            gi._check(gi.lib().rrtmg_sw_mcica_c(C.byref(ah), C.byref(ch)))
        torch.cuda.synchronize()
        e_ms = (time.perf_counter() - t0) * 1e3 / e_steps
        e2e = {"value": sunlit * world / (e_ms / 1e3), "unit": "columns/s", "ms_per_step": e_ms,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e_steps}
        del h, ho

    # roofline: FP32 pipe (no tensor-core contraction in this path)
    m = gi.mcica_subcol_sw(1, min(ncol, 2048), NLAY, 5, 112, 0, c["play"][:2048], c["cldfrac"][:2048],
                           c["ciwp"][:2048], c["clwp"][:2048], c["rei"][:2048], c["rel"][:2048],
                           np.zeros((14, min(ncol, 2048), NLAY)), np.ones((14, min(ncol, 2048), NLAY)),
                           np.zeros((14, min(ncol, 2048), NLAY)), np.zeros((14, min(ncol, 2048), NLAY)),
                           alpha[:2048])
    cloudy = float(m[0].sum() / min(ncol, 2048))
    fl = algorithmic_flops_per_column(NLAY, cloudy)
    peak32 = None
    try:
        torch.backends.cuda.matmul.allow_tf32 = False
        x = torch.randn(8192, 8192, device=dev)
        pk_ms = time_steps(torch, stream, lambda: torch.matmul(x, x), 5, 2)
        peak32 = 2 * 8192 ** 3 / (pk_ms / 1e3) / 1e12
        del x
    except Exception:
        peak32 = None
    achieved = fl * ncol / (ms32 / 1e3) / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    bytes_col = algorithmic_bytes_per_column(NLAY)
    traffic_col = PROFILED_DRAM_BYTES_PER_COLUMN.get(kernel)
    value = sunlit * world / (ms32 / 1e3)

    extra = {}
    if rank == 0 and not args.quick:
        # the headline with aerosols (iaer=10), FP32 and FP64 forms
        from rrtmg_sw_gb300.synthetic import make_columns
        del hc
        torch.cuda.empty_cache()
        ca = make_columns(ncol, NLAY, SEED, clouds=True, lat=True, aerosol=True)
        ha = DevCase(gi, torch, dev, ca, 5, 10, alpha=alpha)
        gi.set_form(gi.FORM_FP32)
        m32a = time_steps(torch, stream, lambda: ha.run(sid), max(3, args.steps // 2), 2)
        r32a = ha.outputs()
        gi.set_form(gi.FORM_FP64)
        m64a = time_steps(torch, stream, lambda: ha.run(sid), 2, 1)
        da = diff_summary(r32a, ha.outputs())
        sa = int((ca["coszen"] > 0).sum())
        extra["headline_iaer10"] = {"fp32": sa / (m32a / 1e3), "fp64": sa / (m64a / 1e3), "speedup": m64a / m32a,
                                    "max_dF_vs_fp64": da["max_dF"], "max_dHR_vs_fp64": da["max_dHR"]}
        del ha, ca, r32a
        torch.cuda.empty_cache()
        extra["clear_1024x60"] = small_workload(gi, torch, dev, sid, "1024x60 clear, icld=0 iaer=0", 1024, 0, 0,
                                                20261203)
        extra["mcica_aer_16384x60"] = small_workload(gi, torch, dev, sid, "16384x60 McICA icld=2 + iaer=10", 16384,
                                                     2, 10, 20261203 + 1)
        extra["batch"] = batch_workload(args, gi, torch, dev, per_instance=False)
        torch.cuda.empty_cache()
        # the adjoint's cost against the forward it differentiates (one timed call each)
        extra["adjoint"] = adjoint_workload(args, gi, k=1, recompute=False)

    line = {
        "metric": METRIC, "value": value, "unit": "columns/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "fused McICA + shortwave solve, %d columns x %d layers per GPU, icld=5 idcor=1, "
                               "inflgsw=2 iceflgsw=3 liqflgsw=1, iaer=0, all sunlit%s" %
                               (ncol, NLAY, ", irng=1 (MT19937 stream in GCM order, generated by jump-ahead "
                                            "segments inside each step)" if args.irng else ""),
                   "ncol": ncol, "nlay": NLAY, "form": "fp32", "kernel": kernel, "l2": None},
        "gpu_launches": args.steps * launches_per_step,
        "clocks": clocks,
    }
    line["config"]["l2"] = "inputs %.2f GB > L2, no flush" % (sum(
        c[k].nbytes for k in ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "cldfrac",
                              "ciwp", "clwp", "rei", "rel")) / 1e9)
    line["roofline"] = {"bound": "fp32", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                        "frac": (achieved / peak32) if peak32 else None,
                        "traffic": traffic_col * ncol if (traffic_col and NLAY == 60) else None,
                        "traffic_source": "ncu dram__bytes_read+write of the solve kernel at 32768 columns, "
                                          "scaled by columns" + ("; its preparation kernel adds %.0f B per column"
                                                                 % PROFILED_PREP_DRAM_BYTES_PER_COLUMN
                                                                 if kernel == "fp32 tiled" else ""),
                        "time_source": "CUDA events over whole steps (the tiled form's step is its preparation "
                                       "kernel, ~6 %, and its solve kernel)",
                        "peak_source": "cuBLAS FP32 (non-TF32) 8192^3 GEMM measured in this run",
                        "flops_per_column": fl, "cloudy_cells_per_column": cloudy}
    line["roofline_hbm"] = {"bound": "hbm", "achieved": bytes_col * ncol / (ms32 / 1e3) / 1e9, "peak": hbm,
                            "unit": "GB/s", "frac": bytes_col * ncol / (ms32 / 1e3) / 1e9 / hbm,
                            "bytes_per_column": bytes_col, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
    line["fp32_counters"] = stats
    if mt_stream is not None:
        line["mt_stream"] = mt_stream
    line.update(extra)
    if ms64 is not None:
        line["fp64"] = {"value": sunlit * world / (ms64 / 1e3), "ms_per_step": ms64,
                        "speedup_fp32_over_fp64": ms64 / ms32, "max_dF_fp32_vs_fp64": d64["max_dF"],
                        "max_dHR_fp32_vs_fp64": d64["max_dHR"]}
    line["e2e"] = e2e
    if rank == 0:
        cores = os.cpu_count() or 1
        if args.quick:
            # a bounded oracle sample: the CPU baseline only
            sample = 32 * cores
            cs = {k: (v[:sample] if isinstance(v, np.ndarray) and v.shape[:1] == (ncol,) else v) for k, v in c.items()}
            _, dt = oracle_solve(cs, 5, 0, alpha=alpha[:sample])
            line["cpu_baseline"] = {"value": sample / dt, "unit": "columns/s", "cores": cores, "kind": "port",
                                    "sample": "%d columns x %d layers, McICA + solve, FP64 oracle, OpenMP" %
                                              (sample, NLAY)}
        else:
            # the FP64 oracle over the whole workload: the CPU baseline, and the
            # FP32 form's error against it per level
            ref, dt = oracle_solve(c, 5, 0, alpha=alpha)  # KISS subcolumns (irng=0)
            line["cpu_baseline"] = {"value": ncol / dt, "unit": "columns/s", "cores": cores, "kind": "port",
                                    "sample": "all %d columns x %d layers, McICA + solve, FP64 oracle, OpenMP, "
                                              "%.0f s" % (ncol, NLAY, dt)}
            if args.irng == 0:
                s32 = diff_summary(res32, ref)
                lv = per_level(res32, ref)
                if ms64 is not None:
                    s64 = diff_summary(res64, ref)
                    line["fp64_vs_oracle"] = {"max_dF": s64["max_dF"], "max_dHR": s64["max_dHR"],
                                              "frac_within_1e-9_rel": s64["frac_within_1e-9_rel"]}
                line["fp32_vs_oracle"] = {"max_dF": s32["max_dF"], "max_dHR": s32["max_dHR"], "max": s32["max"],
                                          "rms": s32["rms"], "per_level_note": "stderr"}
                print(json.dumps({"fp32_vs_oracle_per_level": lv}), file=sys.stderr)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
