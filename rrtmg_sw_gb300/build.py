"""Build ``librrtmg_sw_gb300.so`` for sm_103a with nvcc (no cmake, no torch).

Translation units are compiled in parallel:
  solve_fp64.cu  --fmad=false (plain FP64 form, reference rounding)
  solve_fp32.cu  FMA contraction, approximate FP32 division/sqrt (FP32 form)
  solve_ad.cu    tangent-linear / adjoint of the FP64 form
  mt19937.cu     MT19937 streams with jump-ahead (McICA irng = 1)
  api.cu         host C-ABI
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "librrtmg_sw_gb300.so")
# bounds-check build: every coefficient-table read range-checked into an
# error word (RRTMG_SW_EBOUNDS), for tests; same sources, -DRRTMG_BOUNDS_CHECK
LIB_BC = os.path.join(OUT_DIR, "librrtmg_sw_gb300_bc.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", os.path.join(HERE, "..", "include")]
UNITS = {
    "solve_fp64.cu": ["--fmad=false"],
    "solve_fp32.cu": ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
    "solve_ad.cu": [],
    "mt19937.cu": [],
    "api.cu": [],
}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "rrtmg_sw_gb300.h")]


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False, extra_flags=(), bounds_check=False):
    lib = LIB_BC if bounds_check else LIB
    if not force and up_to_date(lib):
        return lib
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    variant = ["-DRRTMG_BOUNDS_CHECK"] if bounds_check else []
    suffix = "_bc.o" if bounds_check else ".o"

    def compile_one(item):
        src, flags = item
        obj = os.path.join(OUT_DIR, src.replace(".cu", suffix))
        cmd = [cc, *ARCH, *COMMON, *flags, *variant, *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS.items()))
    tmp = lib + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
    print(LIB)
