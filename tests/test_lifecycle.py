"""rrtmg_sw_finalize_c releases the device tables, workspaces, chunk streams
and MT jump tables; entry points then return RRTMG_SW_ENOTINIT until
rrtmg_sw_ini_c runs again, after which results are unchanged bit for bit."""
import ctypes as C

import numpy as np
import pytest

from rrtmg_sw_gb300 import interface as gi
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

pytestmark = pytest.mark.gpu


def test_finalize_and_reinit():
    torch = pytest.importorskip("torch")
    from rrtmg_sw_gb300 import build
    build.build()
    gi.rrtmg_sw_ini(1.004e3)
    gi.set_form(gi.FORM_FP64)
    c = make_columns(33, 47, 77, clouds=True)
    kw = gcm_inputs(c, icld=2, iaer=0)
    cl = dict(permuteseed=112, irng=0, cldfrac=c["cldfrac"], ciwp=c["ciwp"], clwp=c["clwp"], rei=c["rei"],
              rel=c["rel"])
    r1 = gi.rrtmg_sw(**kw, clouds=cl, extra=True)
    buf = torch.empty(100_003, dtype=torch.int32, device="cuda")
    gi.mt_stream_dev(5, buf.numel(), buf.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
    m1 = buf.cpu().numpy().copy()
    assert gi.lib().rrtmg_sw_finalize_c() == 0
    a = gi.RrtmgSwArgs()
    a.ncol, a.nlay = 4, 47
    assert gi.lib().rrtmg_sw_c(C.byref(a)) == 1  # RRTMG_SW_ENOTINIT
    gi.rrtmg_sw_ini(1.004e3)
    r2 = gi.rrtmg_sw(**kw, clouds=cl, extra=True)
    buf.zero_()
    gi.mt_stream_dev(5, buf.numel(), buf.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
    assert np.array_equal(buf.cpu().numpy(), m1)
    for k in r1:
        assert np.array_equal(r1[k], r2[k]), k
