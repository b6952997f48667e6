"""GB300 (sm_103a) implementation of the RRTMG_SW shortwave column solve.

The compute path is ``librrtmg_sw_gb300.so`` (hand-written CUDA kernels
behind a C ABI, include/rrtmg_sw_gb300.h); :mod:`rrtmg_sw_gb300.interface`
mirrors the reference's GCM interface on top of it.
"""
from .interface import (FORM_FP32, FORM_FP64, NBNDSW, NGPTSW, RRTMGError, get_alpha,  # noqa: F401
                       mcica_subcol_sw, rrtmg_sw, rrtmg_sw_ini, set_form)
