"""CPU-only checks of the C ABI library: it builds, loads, and exports every
entry point declared in include/rrtmg_sw_gb300.h (no compute calls)."""
import ctypes
import os
import re

import numpy as np

from rrtmg_sw_gb300 import build, interface
from rrtmg_sw_gb300.synthetic import make_columns

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rrtmg_sw_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*\**\s*(\w+_c)\s*\(", text)))


def test_library_exports_all_declared_symbols():
    build.build()
    lib = ctypes.CDLL(interface.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


STRUCTS = (("rrtmg_sw_args", interface.RrtmgSwArgs), ("rrtmg_sw_clouds", interface.RrtmgSwClouds),
           ("rrtmg_sw_ad_args", interface.RrtmgSwAdArgs))


def header_fields(struct):
    """(name, C type) of every field of ``struct`` in include/rrtmg_sw_gb300.h, in order."""
    text = open(os.path.join(ROOT, "include", "rrtmg_sw_gb300.h")).read()
    body = text[text.index("typedef struct %s {" % struct):text.index("} %s;" % struct)]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S).split("{", 1)[1]
    out = []
    for decl in body.split(";")[:-1]:
        decl = " ".join(decl.split())
        m = re.match(r"((?:const\s+)?\w+)\s*(.*)", decl)
        base, rest = m.group(1), m.group(2)
        for item in rest.split(","):
            item = item.strip()
            ptr = item.startswith("*")
            out.append((item.lstrip("*").strip(), base.replace("const ", "") + ("*" if ptr else "")))
    return out


def test_struct_fields_match_ctypes_names_and_order():
    for struct, cls in STRUCTS:
        names = [n for n, _ in header_fields(struct)]
        assert names == [f[0] for f in cls._fields_], struct


def c_layout(struct):
    """(offset, size) of each field and sizeof(struct), from a probe compiled
    with the system C compiler against the header."""
    import shutil
    import subprocess
    import tempfile
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    fields = header_fields(struct)
    src = ["#include <stddef.h>", "#include <stdio.h>", '#include "rrtmg_sw_gb300.h"', "int main(void) {"]
    for n, _ in fields:
        src.append('  printf("%%zu %%zu\\n", offsetof(%s, %s), sizeof(((%s *)0)->%s));' % (struct, n, struct, n))
    src.append('  printf("%%zu\\n", sizeof(%s));' % struct)
    src.append("  return 0;\n}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(src) + "\n")
        exe = os.path.join(d, "probe")
        subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), c, "-o", exe],
                       check=True)
        lines = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    offs = [tuple(int(x) for x in l.split()) for l in lines[:len(fields)]]
    return fields, offs, int(lines[len(fields)])


def test_struct_layout_matches_c_compiler():
    # offsets and sizes as a C compiler lays the header's structs out, against
    # the ctypes mirror the Python interface passes to the library
    import ctypes as C
    for struct, cls in STRUCTS:
        fields, offs, size = c_layout(struct)
        for (n, _), (o, sz) in zip(fields, offs):
            f = getattr(cls, n)
            assert (f.offset, f.size) == (o, sz), (struct, n, (f.offset, f.size), (o, sz))
        assert C.sizeof(cls) == size, struct


def shim_type_fields(struct):
    """(name, kind) of the components of the Fortran shim's bind(c) type ``struct``."""
    text = open(os.path.join(ROOT, "rrtmg_sw_gb300", "fortran", "rrtmg_sw_gb300_shim.f90")).read()
    body = text[text.index("type, bind(c) :: %s" % struct):text.index("end type %s" % struct)]
    out = []
    for line in body.split("\n")[1:]:
        line = line.split("!")[0].strip()
        if "::" not in line:
            continue
        kind, names = [x.strip() for x in line.split("::")]
        for n in names.split(","):
            out.append((n.strip(), kind))
    return out


def test_fortran_shim_types_match_header():
    # every field of the C structs, in order, with the interoperable kind of
    # its C type (pointer -> type(c_ptr), int32_t -> integer(c_int32_t),
    # double -> real(c_double))
    kinds = {"int32_t": "integer(c_int32_t)", "double": "real(c_double)"}
    for struct in ("rrtmg_sw_args", "rrtmg_sw_clouds"):
        want = [(n, "type(c_ptr)" if t.endswith("*") else kinds[t]) for n, t in header_fields(struct)]
        assert shim_type_fields(struct) == want, struct


def test_errstr_without_gpu():
    build.build()
    lib = interface.lib()
    assert lib.rrtmg_sw_errstr_c(12).decode() == "ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS"
    assert lib.rrtmg_sw_errstr_c(21).decode().startswith("MCICA_SUBCOL: KISSVEC SEED GENERATOR")


def test_synthetic_columns_are_monotonic_and_bounded():
    c = make_columns(200, 60, 20261203, clouds=True, aerosol=True)
    assert np.all(np.diff(c["plev"], axis=1) < 0)
    assert np.all(c["play"] < c["plev"][:, :-1]) and np.all(c["play"] > c["plev"][:, 1:])
    assert c["h2ovmr"].min() >= 3e-6
    assert 0.1 <= c["cldfrac"][c["cldfrac"] > 0].min() and c["cldfrac"].max() <= 1.0
    assert c["rei"].min() >= 5.0 and c["rei"].max() <= 140.0
    assert c["rel"].min() >= 2.5 and c["rel"].max() <= 60.0
