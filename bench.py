"""Benchmark: sunlit columns/s of the fused McICA shortwave solve on one GB300.

Workload (N=1): 262,144 columns x 60 layers, McICA clouds with
exponential-random overlap (icld=5, idcor=1, KISS subcolumns generated in
the kernel), inflgsw=2/iceflgsw=3/liqflgsw=1, no aerosol, all columns
sunlit.  A step is one call of the fused entry point over the whole batch.

value   : FP32-form sunlit columns/s, kernel only, inputs resident in HBM
          (inputs are ~1.6 GB, larger than L2, so no flush is needed)
e2e     : the same through the host-array C-ABI entry point
          (rrtmg_sw_mcica_c): H2D of the inputs from pinned memory, the
          solve, D2H of the six output arrays, every step
fp64    : the plain FP64 form on the same inputs (the metric's comparison)

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


# DRAM bytes per column of k_solve<float> measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum) in a full capture at 32768 columns x 60 layers; the traffic is
# per column pair, so a launch's traffic scales with its columns.
PROFILED_DRAM_BYTES_PER_COLUMN = 28.38e9 / 32768


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
    """48 ragged instances (ncol log-uniform in 512..131072, nlay from
    {40,47,60,72,91,137}, 40 % night columns, McICA clouds icld=2 with
    inflgsw=2/iceflgsw=3/liqflgsw=1, FP64 form) in one persistent launch
    replayed from a CUDA graph; per-instance figures from single calls."""
    import torch
    from rrtmg_sw_gb300 import build, interface as gi
    from rrtmg_sw_gb300.synthetic import make_columns
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    fp32 = args.batch_form == "fp32"
    form_name = "FP32 form" if fp32 else "FP64 form"
    gi.set_form(gi.FORM_FP32 if fp32 else gi.FORM_FP64)
    rng = np.random.default_rng(20261203 + 2)
    dev = torch.device("cuda", 0)
    ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), gi._dp)
    insts = []
    for i in range(args.instances):
        ncol = int(round(np.exp(rng.uniform(np.log(512), np.log(131072)))))
        nlay = int(rng.choice([40, 47, 60, 72, 91, 137]))
        c = make_columns(ncol, nlay, 20261203 + 2 + 1000 * i, clouds=True, night_frac=0.4)
        T = lambda x: torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).to(dev)
        t = {k: T(c[k]) for k in ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir",
                                  "asdif", "aldir", "aldif", "coszen", "cldfrac", "ciwp", "clwp", "rei", "rel")}
        for k in ("swuflx", "swdflx", "swuflxc", "swdflxc"):
            t[k] = torch.empty(ncol * (nlay + 1), dtype=torch.float64, device=dev)
        for k in ("swhr", "swhrc"):
            t[k] = torch.empty(ncol * nlay, dtype=torch.float64, device=dev)
        a = gi.RrtmgSwArgs()
        a.ncol, a.nlay, a.icld, a.iaer = ncol, nlay, 2, 0
        for k in ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif", "aldir",
                  "aldif", "coszen", "swuflx", "swdflx", "swuflxc", "swdflxc", "swhr", "swhrc"):
            setattr(a, k, ptr(t[k]))
        a.adjes, a.dyofyr, a.scon, a.isolvar = 1.0, 0, 1360.85, 0
        a.inflgsw, a.iceflgsw, a.liqflgsw = 2, 3, 1
        a.idelm = 1
        cl = gi.RrtmgSwClouds()
        cl.permuteseed, cl.irng = 112, 0
        for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
            setattr(cl, k, ptr(t[k]))
        insts.append(dict(t=t, a=a, c=cl, ncol=ncol, nlay=nlay, sunlit=int((c["coszen"] > 0).sum())))
    stream = torch.cuda.current_stream(dev)
    sid = stream.cuda_stream
    plan = gi.BatchPlan([x["a"] for x in insts], [x["c"] for x in insts], stream=sid)
    for _ in range(max(1, args.warmup - 1)):
        plan.run(sid)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(1, args.steps // 5)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        plan.run(sid)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    sunlit = sum(x["sunlit"] for x in insts)
    per = []
    for x in insts:  # each instance alone through rrtmg_sw_mcica_dev_c
        gi.rrtmg_sw_dev(x["a"], sid, x["c"])
        torch.cuda.synchronize()
        e0.record(stream)
        gi.rrtmg_sw_dev(x["a"], sid, x["c"])
        e1.record(stream)
        torch.cuda.synchronize()
        m1 = e0.elapsed_time(e1)
        per.append({"ncol": x["ncol"], "nlay": x["nlay"], "sunlit": x["sunlit"], "single_ms": m1,
                    "single_columns_per_s": x["sunlit"] / (m1 / 1e3)})
    info = plan.info()
    plan.close()
    line = {"metric": "sunlit columns/s, 48 ragged instances in one persistent launch (%s)" % form_name,
            "value": sunlit / (ms / 1e3), "unit": "columns/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if fp32 else "f64", "data": "synthetic",
            "config": {"workload": "%d instances, ncol log-uniform 512..131072, nlay in {40,47,60,72,91,137}, 40%% "
                                   "night, McICA icld=2, %s" % (len(insts), form_name),
                       "columns": sum(x["ncol"] for x in insts), "sunlit": sunlit},
            "sum_of_single_calls_ms": sum(p["single_ms"] for p in per),
            "autotuner": info, "instances": per}
    print(json.dumps(line))


def run_adjoint(args):
    """Adjoint cost: 65536 columns x 60 layers, McICA clouds (icld=2, masks
    frozen), objective TOA up + surface net + heating-rate sum; forward,
    tangent-linear and adjoint (stored / recomputed local Jacobians) through
    the host-array C ABI, each timed end to end."""
    from rrtmg_sw_gb300 import build, interface as gi
    from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    gi.set_form(gi.FORM_FP64)
    ncol = args.ncol if args.ncol != NCOL else 65536
    c = make_columns(ncol, NLAY, 20261203 + 4, clouds=True)
    kw = gcm_inputs(c, icld=2, iaer=0)
    for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl"):
        kw[k] = None  # fused McICA: the subcolumn arrays are not passed
    cl = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
              rel=c["rel"])
    w = (1.0, 1.0, 1.0)

    def best(f, k=3):
        f()
        ts = []
        for _ in range(k):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        return min(ts) * 1e3

    fwd = best(lambda: gi.rrtmg_sw(**kw, clouds=cl))
    d = {k: np.ones_like(kw["tlay"]) for k in gi.AD_LAYER}
    tl = best(lambda: gi.rrtmg_sw_tl(kw, d, cl, w))
    ad_s = best(lambda: gi.rrtmg_sw_ad(kw, cl, w, store=True))
    ad_r = best(lambda: gi.rrtmg_sw_ad(kw, cl, w, store=False))
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    slot = lambda fields: ((NLAY + 1) * fields * 224 + 2 * 15 * NLAY * 4) * 8
    line = {"metric": "adjoint cost relative to the FP64 forward (host-array calls, end to end)",
            "value": ad_s / fwd, "unit": "x forward", "n_gpus": 1, "higher_is_better": False,
            "config": {"workload": "%d columns x %d layers, McICA icld=2, objective TOA up + sfc net + HR sum"
                                   % (ncol, NLAY)},
            "forward_fp64_ms": fwd, "tangent_linear_ms": tl, "adjoint_store_ms": ad_s, "adjoint_recompute_ms": ad_r,
            "scratch_bytes_store": slot(45) * sms, "scratch_bytes_recompute": slot(20) * sms}
    print(json.dumps(line))


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
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    # alpha for icld=5/idcor=1 on the device (get_alpha)
    alpha = gi.get_alpha(1, ncol, NLAY, 5, 1, 0.0, c["dz"], c["lat"], 94, c["cldfrac"])
    dev = torch.device("cuda", local)

    def T(x):
        return torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).to(dev)

    d = {k: T(c[k]) for k in ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr",
                              "asdir", "asdif", "aldir", "aldif", "coszen", "cldfrac", "ciwp", "clwp", "rei", "rel")}
    d["alpha"] = T(alpha)
    outs = {k: torch.empty(ncol * (NLAY + 1), dtype=torch.float64, device=dev)
            for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    outs.update({k: torch.empty(ncol * NLAY, dtype=torch.float64, device=dev) for k in ("swhr", "swhrc")})
    a = gi.RrtmgSwArgs()
    a.ncol, a.nlay, a.icld, a.iaer = ncol, NLAY, 5, 0
    ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), gi._dp)
    for k in ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif", "aldir",
              "aldif", "coszen"):
        setattr(a, k, ptr(d[k]))
    a.adjes, a.dyofyr, a.scon, a.isolvar = 1.0, 0, 1360.85, 0
    a.inflgsw, a.iceflgsw, a.liqflgsw = 2, 3, 1
    for k, v in outs.items():
        setattr(a, k, ptr(v))
    a.idelm = 1
    cl = gi.RrtmgSwClouds()
    cl.permuteseed, cl.irng = 112, args.irng
    for k in ("cldfrac", "ciwp", "clwp", "rei", "rel", "alpha"):
        setattr(cl, k, ptr(d[k]))
    stream = torch.cuda.current_stream(dev)
    sid = stream.cuda_stream

    def step():
        gi.rrtmg_sw_dev(a, sid, cl)

    def timed(form, steps, warmup):
        gi.set_form(form)
        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    import tempfile
    clk_path = os.path.join(tempfile.gettempdir(), "rrtmg_sw_bench_clocks_%d.csv" % os.getpid())
    with Clocks(clk_path) as clk:
        ms32 = timed(gi.FORM_FP32, args.steps, args.warmup)
    clocks = clk.summary()
    res32 = {k: v.cpu().numpy() for k, v in outs.items()}
    sunlit = int((c["coszen"] > 0).sum())
    ms64 = None
    if not args.no_fp64:
        ms64 = timed(gi.FORM_FP64, max(2, args.steps // 5), 1)
        res64 = {k: v.cpu().numpy() for k, v in outs.items()}
        err = {k: float(np.max(np.abs(res32[k] - res64[k]))) for k in res32}
        rms = {k: float(np.sqrt(np.mean((res32[k] - res64[k]) ** 2))) for k in res32}
        # per level (fluxes, surface first) / per layer (heating rates): max and RMS over columns
        per_level = {}
        for k in res32:
            nl = NLAY if k in ("swhr", "swhrc") else NLAY + 1
            dk = (res32[k] - res64[k]).reshape((nl, ncol))
            per_level[k] = {"max": [float("%.3g" % v) for v in np.max(np.abs(dk), axis=1)],
                            "rms": [float("%.3g" % v) for v in np.sqrt(np.mean(dk * dk, axis=1))]}
    gi.set_form(gi.FORM_FP32)

    # irng = 1: the MT19937 generator alone on the call's stream (icld 5: two draws per cell)
    mt_stream = None
    if args.irng == 1:
        nmt = 2 * 112 * ncol * NLAY
        buf = torch.empty(nmt, dtype=torch.int32, device=dev)
        gi.mt_stream_dev(112, nmt, buf.data_ptr(), 0, sid)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            gi.mt_stream_dev(112, nmt, buf.data_ptr(), 0, sid)
        e1.record(stream)
        torch.cuda.synchronize()
        mt_ms = e0.elapsed_time(e1) / 3
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
        ho = {k: torch.empty(v.numel(), dtype=torch.float64).pin_memory() for k, v in outs.items()}
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

    # roofline: FP32 pipe (no tensor-core contraction in this path)
    cloudy = float(os.environ.get("RRTMG_CLOUDY_CELLS", "0"))
    if cloudy == 0.0:
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
        for _ in range(2):
            torch.matmul(x, x)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            torch.matmul(x, x)
        e1.record()
        torch.cuda.synchronize()
        peak32 = 2 * 8192 ** 3 * 5 / (e0.elapsed_time(e1) / 1e3) / 1e12
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
    value = sunlit * world / (ms32 / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "columns/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "fused McICA + shortwave solve, %d columns x %d layers per GPU, icld=5 idcor=1, "
                               "inflgsw=2 iceflgsw=3 liqflgsw=1, iaer=0, all sunlit%s" %
                               (ncol, NLAY, ", irng=1 (MT19937 stream in GCM order, generated by jump-ahead "
                                            "segments inside each step)" if args.irng else ""),
                   "ncol": ncol, "nlay": NLAY, "form": "fp32", "l2": "inputs %.2f GB > L2, no flush" %
                   (sum(v.numel() * 8 for v in d.values()) / 1e9)},
        "fp64": None if ms64 is None else {"value": sunlit * world / (ms64 / 1e3), "ms_per_step": ms64,
                                           "speedup_fp32_over_fp64": ms64 / ms32,
                                           "max_abs_diff_fp32_vs_fp64": err, "rms_diff_fp32_vs_fp64": rms,
                                           "per_level_diff_fp32_vs_fp64": per_level},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                     "frac": (achieved / peak32) if peak32 else None,
                     "traffic": PROFILED_DRAM_BYTES_PER_COLUMN * ncol if NLAY == 60 else None,
                     "traffic_unit": "bytes per launch (ncu capture at 32768 columns, scaled by columns)",
                     "peak_source": "cuBLAS FP32 (non-TF32) 8192^3 GEMM measured in this run",
                     "flops_per_column": fl, "cloudy_cells_per_column": cloudy},
        "roofline_hbm": {"bound": "hbm", "achieved": bytes_col * ncol / (ms32 / 1e3) / 1e9, "peak": hbm,
                         "unit": "GB/s", "frac": bytes_col * ncol / (ms32 / 1e3) / 1e9 / hbm,
                         "bytes_per_column": bytes_col, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "e2e": e2e,
        "gpu_launches": args.steps * (3 if args.irng else 1),
        "clocks": clocks,
    }
    if mt_stream is not None:
        line["mt_stream"] = mt_stream
    if rank == 0:
        cores = os.cpu_count() or 1
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import pyoracle
            from rrtmg_sw_gb300.synthetic import gcm_inputs
            sample = 32 * cores
            cs = inputs(sample, SEED)
            al = pyoracle.get_alpha(sample, NLAY, 5, 1, 0.0, cs["dz"].ravel(order="F"), cs["lat"], 94,
                                    cs["cldfrac"].ravel(order="F"))
            z14 = np.zeros(14 * sample * NLAY)
            t0 = time.perf_counter()
            mm = pyoracle.mcica_subcol_sw(sample, NLAY, 5, 112, args.irng, *(cs[k].ravel(order="F") for k in
                                                                     ("play", "cldfrac", "ciwp", "clwp", "rei",
                                                                      "rel")), z14, z14 + 1.0, z14, z14, al)
            names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl",
                     "fsfcmcl")
            kw = gcm_inputs(cs, icld=5, iaer=0, mcica=tuple(mm[k] for k in names))
            inp = {k: kw[k] for k in pyoracle.GCM_INPUTS + pyoracle.MCICA_INPUTS + pyoracle.AER_INPUTS}
            pyoracle.rrtmg_sw(sample, NLAY, 5, 0, inp, nthreads=cores)
            dt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": sample / dt, "unit": "columns/s", "cores": cores, "kind": "port",
                                    "sample": "%d columns x %d layers, McICA + solve, FP64 oracle, OpenMP" %
                                              (sample, NLAY)}
        except Exception as ex:  # the baseline is reported, not required
            line["cpu_baseline"] = {"value": None, "unit": "columns/s", "cores": cores, "kind": "port",
                                    "sample": "failed: %s" % ex}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
