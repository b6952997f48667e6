"""Native callers of the library: a C program that includes
include/rrtmg_sw_gb300.h, and a Fortran GCM-style program built on the
ISO_C_BINDING shim (rrtmg_sw_gb300/fortran/rrtmg_sw_gb300_shim.f90) that
keeps RRTMG_SW's module and routine names and argument lists
(rrtmg_sw_rad.f90:99-111, mcica_subcol_gen_sw.f90:181-185,
rrtmg_sw_init.f90:47).  Both are compiled on the machine that runs the test
and checked against the Python (ctypes) calls of the same entry points on
the same inputs.  Tolerance 0: the same library on the same inputs gives the
same bits whichever language calls it.

The Fortran program passes arrays whose leading dimension (pcols) exceeds
ncol, as GCM physics buffers do, so the shim's packing path runs; the
padding columns hold values that would poison any result they leaked into.
It is built twice, the second time with the reference's -i8 -r8 default
kinds (gfortran -fdefault-integer-8 -fdefault-real-8).  Skipped when no
Fortran compiler is installed.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from rrtmg_sw_gb300 import interface as gpu
from rrtmg_sw_gb300.synthetic import gcm_inputs, make_columns

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.dirname(gpu.LIB_PATH)
OUTS = ("swuflx", "swdflx", "swhr", "swuflxc", "swdflxc", "swhrc")


@pytest.fixture(scope="module", autouse=True)
def _init():
    from rrtmg_sw_gb300 import build
    build.build()
    gpu.rrtmg_sw_ini(1.004e3)
    gpu.set_form(gpu.FORM_FP64)


def split_outputs(buf, ncol, nlay):
    res, o = {}, 0
    for k in OUTS:
        n = ncol * (nlay if k in ("swhr", "swhrc") else nlay + 1)
        res[k] = buf[o:o + n].reshape((ncol, -1), order="F")
        o += n
    return res, o


def test_c_program_through_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "abi_driver"
    subprocess.run([cc, "-O2", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_driver.c"), "-o", str(exe), "-L", LIBDIR,
                    "-lrrtmg_sw_gb300", "-Wl,-rpath," + LIBDIR], check=True)
    c = make_columns(9, 60, 20261216)
    ncol, nlay = 9, 60
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([ncol, nlay], dtype=np.int32).tofile(f)
        for k in ("play", "plev", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "o2vmr", "asdir", "asdif",
                  "aldir", "aldif", "coszen"):
            np.asfortranarray(c[k]).ravel(order="F").astype(np.float64).tofile(f)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    raw = open(tmp_path / "out.bin", "rb").read()
    size = np.frombuffer(raw[:8], dtype=np.int64)[0]
    rc = np.frombuffer(raw[8:12], dtype=np.int32)[0]
    assert rc == 0
    assert size == C.sizeof(gpu.RrtmgSwArgs)
    got, _ = split_outputs(np.frombuffer(raw[12:], dtype=np.float64), ncol, nlay)
    ref = gpu.rrtmg_sw(**gcm_inputs(c, icld=0, iaer=0))
    for k, v in zip(OUTS, ref):
        np.testing.assert_array_equal(got[k], v, err_msg=k)


def build_fortran(fc, tmp_path, tag, flags):
    d = tmp_path / tag
    d.mkdir()
    shim = os.path.join(ROOT, "rrtmg_sw_gb300", "fortran", "rrtmg_sw_gb300_shim.f90")
    drv = os.path.join(ROOT, "tests", "fortran", "shim_driver.f90")
    subprocess.run([fc, "-O2", "-std=f2008", *flags, "-J", str(d), "-c", shim, "-o", str(d / "shim.o")], check=True)
    exe = d / "shim_driver"
    subprocess.run([fc, "-O2", *flags, "-I", str(d), drv, str(d / "shim.o"), "-o", str(exe), "-L", LIBDIR,
                    "-lrrtmg_sw_gb300", "-Wl,-rpath," + LIBDIR], check=True)
    return exe


@pytest.mark.parametrize("flags", [[], ["-fdefault-integer-8", "-fdefault-real-8"]], ids=["default", "i8r8"])
def test_fortran_gcm_program_through_shim(tmp_path, flags):
    fc = shutil.which("gfortran")
    if fc is None:
        pytest.skip("no Fortran compiler (gfortran) on this machine")
    exe = build_fortran(fc, tmp_path, "i8r8" if flags else "default", flags)
    ncol, nlay, pcols = 7, 60, 10
    c = make_columns(ncol, nlay, 20261217, clouds=True)

    def padded(x):
        x = np.asarray(x)
        if x.ndim == 1:
            y = np.full(pcols, 1.0e30)
            y[:ncol] = x
            return y
        y = np.full((pcols,) + x.shape[1:], 1.0e30)
        y[:ncol] = x
        return y

    order = ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
             "asdir", "asdif", "aldir", "aldif", "coszen")
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([ncol, nlay, pcols], dtype=np.int32).tofile(f)
        for k in order + ("cldfrac", "ciwp", "clwp", "rei", "rel"):
            padded(c[k]).ravel(order="F").tofile(f)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    raw = np.fromfile(tmp_path / "out.bin", dtype=np.uint8)
    sizes = np.frombuffer(raw[:16].tobytes(), dtype=np.int64)
    assert sizes[0] == C.sizeof(gpu.RrtmgSwArgs) and sizes[1] == C.sizeof(gpu.RrtmgSwClouds)
    vals = np.frombuffer(raw[16:].tobytes(), dtype=np.float64)
    clear, n = split_outputs(vals, ncol, nlay)
    cloudy, _ = split_outputs(vals[n:], ncol, nlay)
    ref_clear = gpu.rrtmg_sw(**gcm_inputs(c, icld=0, iaer=0))
    z = np.zeros((14, ncol, nlay))
    m = gpu.mcica_subcol_sw(1, ncol, nlay, 2, 112, 0, c["play"], c["cldfrac"], c["ciwp"], c["clwp"], c["rei"],
                            c["rel"], z, z + 1.0, z, z, None)
    ref_cloudy = gpu.rrtmg_sw(**gcm_inputs(c, icld=2, iaer=0, mcica=m))
    for k, a, b in zip(OUTS, ref_clear, ref_cloudy):
        np.testing.assert_array_equal(clear[k], a, err_msg="clear " + k)
        np.testing.assert_array_equal(cloudy[k], b, err_msg="mcica " + k)
