"""Bounds-check build (-DRRTMG_BOUNDS_CHECK): every coefficient-table read
is range-checked against the blob and a violation returns RRTMG_SW_EBOUNDS.
The cases of bounds_cases.py (every form, overlap, RNG, aerosol and cloud
option, non-McICA, extra and per-band outputs, adjoint) must run clean, and
its FP64-form results must equal the normal build's bit for bit (the checks
add no arithmetic; the adjoint, whose gradient sums use atomics, to 1e-8 of
each field's largest entry); FP32-form results within 1e-3 W m-2 / K d-1."""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

pytestmark = pytest.mark.gpu


def test_bounds_check_build_runs_clean(tmp_path):
    from rrtmg_sw_gb300 import build
    build.build()
    lib_bc = build.build(bounds_check=True)
    out = str(tmp_path / "bc.npz")
    env = dict(os.environ, RRTMG_SW_LIB=lib_bc, PYTHONPATH=os.pathsep.join([ROOT, os.path.join(ROOT, "oracle")]))
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_cases.py"), out], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    bc = np.load(out)
    sys.path.insert(0, HERE)
    import bounds_cases
    ref = bounds_cases.run()
    assert set(ref) == set(bc.files)
    for k, v in ref.items():
        if k.startswith("f32"):
            assert np.max(np.abs(bc[k] - v)) <= 1e-3, k
        elif k.startswith("ad_"):
            # the adjoint unit contracts FMAs and sums gradients with shared-memory
            # atomics (order varies): compare to 1e-8 of the field's largest entry
            assert np.max(np.abs(bc[k] - v)) <= 1e-8 * max(np.max(np.abs(v)), 1e-300), k
        else:
            assert np.array_equal(bc[k], v), k
