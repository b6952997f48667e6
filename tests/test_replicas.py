"""Multi-process path on the CPU (gloo, world size 2).

Columns are independent, so N GPUs run N replicas: each rank solves its own
columns and nothing is exchanged on the data path.  These tests check the
host logic that makes that sound, without a GPU:
  - two gloo ranks each solve half of a column set with the FP64 oracle
    (KISS McICA, per-column streams) and rank 0 gathers them: the result
    equals one process solving all columns, bit for bit;
  - the MT19937 GCM-order stream split at a rank boundary: rank 1 starts at
    its offset through the host jump-ahead and continues the sequence that
    one process would draw;
  - bench.py's reference arm under torchrun with two ranks prints exactly
    one JSON line (rank 0) and both ranks exit 0.
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
NCOL, NLAY = 64, 40


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def solve(c, cols):
    import pyoracle
    from rrtmg_sw_gb300.synthetic import gcm_inputs
    sub = {k: (v[cols] if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == NCOL else v)
           for k, v in c.items()}
    n = len(cols)
    m = pyoracle.mcica_subcol_sw(n, NLAY, 2, 112, 0, *(sub[k].ravel(order="F") for k in
                                                       ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")),
                                 np.zeros(14 * n * NLAY), np.ones(14 * n * NLAY), np.zeros(14 * n * NLAY),
                                 np.zeros(14 * n * NLAY), np.zeros(n * NLAY))
    names = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")
    kw = gcm_inputs(sub, icld=2, iaer=0, mcica=tuple(m[k] for k in names))
    inp = {k: kw[k] for k in pyoracle.GCM_INPUTS + pyoracle.MCICA_INPUTS}
    out = pyoracle.rrtmg_sw(n, NLAY, 2, 0, inp, nthreads=1)
    return np.concatenate([out[k].reshape((n, -1), order="F") for k in sorted(out)], axis=1)


def rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from rrtmg_sw_gb300.synthetic import make_columns
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    pyoracle.init(1.004e3)
    c = make_columns(NCOL, NLAY, 20261212, clouds=True)
    per = NCOL // world
    mine = torch.from_numpy(solve(c, np.arange(rank * per, (rank + 1) * per)))
    parts = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine)
    if rank == 0:
        q.put(torch.cat(parts).numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process():
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from rrtmg_sw_gb300.synthetic import make_columns
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    pyoracle.init(1.004e3)
    ref = solve(make_columns(NCOL, NLAY, 20261212, clouds=True), np.arange(NCOL))
    assert np.array_equal(got, ref)


def test_mt_stream_split_at_rank_boundary():
    # one GCM-order stream of 2 * 112 * NCOL * NLAY draws (icld 5) cut in two:
    # rank 1's first window from the jump equals the words one process draws there
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from rrtmg_sw_gb300 import interface as gi
    n = 2 * 112 * NCOL * NLAY
    seq = pyoracle.mt_real(224, n)
    for off in (n // 2, n // 2 + 1, n - 624):
        w = gi.mt_temper(gi.mt_window(224, off)).astype(np.float64) / 4294967295.0
        assert np.array_equal(w, seq[off:off + 624]), off


def test_reference_arm_under_torchrun_two_ranks():
    env = dict(os.environ, RRTMG_REF_SAMPLE="64", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
