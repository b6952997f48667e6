"""Build ``rrtmg_sw_tables.bin``: the RRTMG_SW coefficient tables as plain FP64 data.

This is a build step, run once on a machine that has the RRTMG_SW source tree
(``python extract_tables.py <path-to-RRTMG_SW>``); its output is committed so
that nothing at run time needs the Fortran sources.

What it does, and where each step comes from:

* parses the numeric array constructors of the 224-g-point k-distribution
  data (``src/rrtmg_sw_k_g.f90`` subroutines ``sw_kgb16`` .. ``sw_kgb29``,
  shapes from ``modules/rrsw_kg16.f90`` .. ``rrsw_kg29.f90``), including the
  band-29 irradiance rescaling at ``rrtmg_sw_k_g.f90:62460-62461``;
* parses the g-point mapping (``src/rrtmg_sw_init.f90:263-386``, ``swcmbdat``),
  aerosol (``swaerpr`` ``:389-489``) and cloud (``swcldpr`` ``:1692-3514``) data
  and the reference atmosphere (``src/rrtmg_sw_setcoef.f90:308-362``);
* performs the 224 -> 112 g-point reduction of ``rrtmg_sw_ini``
  (weights ``rrtmg_sw_init.f90:130-154``, band reductions ``cmbgb16s`` ..
  ``cmbgb29`` ``:492-1689``): absorption-like quantities are combined with the
  ``rwgt`` weights, solar-source quantities (``sfluxref``, ``irradnce``,
  ``facbrght``, ``snsptdrk``) are plain sums.  Sums are accumulated in the same
  order as the reference loops, one FP64 rounding per multiply and per add.

File format (little endian): magic ``RRSWTB01``, ``u32`` record count, then per
record a 32-byte NUL-padded name, ``u32`` ndim, ``u32 dims[4]`` (Fortran shape,
column-major, unused dims = 1), ``u64`` element count and the FP64 values in
Fortran (column-major) order.
"""
import os
import re
import struct
import sys

import numpy as np

BANDS = list(range(16, 30))
NG = {16: 6, 17: 12, 18: 8, 19: 8, 20: 10, 21: 10, 22: 2, 23: 10, 24: 8,
      25: 6, 26: 6, 27: 8, 28: 6, 29: 12}
SOURCE_NAMES = {"sfluxrefo", "irradnceo", "facbrghto", "snsptdrko"}


def _strip_comment(line):
    out = []
    in_str = None
    for ch in line:
        if in_str:
            out.append(ch)
            if ch == in_str:
                in_str = None
        elif ch in "'\"":
            in_str = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def statements(text):
    """Yield (subroutine, statement) pairs with continuations joined."""
    sub = None
    buf = ""
    for raw in text.splitlines():
        line = _strip_comment(raw).rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if s.startswith("&"):
            s = s[1:]
        if buf:
            buf += " " + s
        else:
            buf = s
        if buf.endswith("&"):
            buf = buf[:-1]
            continue
        stmt = buf.strip()
        buf = ""
        m = re.match(r"(?i)^subroutine\s+(\w+)", stmt)
        if m:
            sub = m.group(1).lower()
        yield sub, stmt


def parse_number(tok):
    tok = tok.strip()
    tok = re.sub(r"_rb$", "", tok)
    tok = re.sub(r"_im$", "", tok)
    return float(tok.replace("d", "e").replace("D", "e"))


def parse_values(rhs):
    rhs = rhs.strip()
    if rhs.startswith("(/"):
        body = rhs[2:rhs.rindex("/)")]
        return [parse_number(t) for t in body.split(",") if t.strip()]
    return [parse_number(rhs)]


class FArray:
    """A Fortran array with explicit lower/upper bounds, column-major."""

    def __init__(self, bounds):
        self.bounds = bounds  # list of (lo, hi)
        self.shape = [hi - lo + 1 for lo, hi in bounds]
        self.data = np.full(self.shape, np.nan, order="F")

    def assign(self, subs, values):
        idx = []
        free = []
        for d, sub in enumerate(subs):
            sub = sub.strip()
            lo, hi = self.bounds[d]
            if sub == ":":
                idx.append(slice(None))
                free.append(d)
            else:
                idx.append(int(sub) - lo)
        target = self.data[tuple(idx)]
        n = int(np.prod([self.shape[d] for d in free])) if free else 1
        if len(values) != n:
            raise ValueError("value count %d != section size %d" % (len(values), n))
        arr = np.array(values, dtype=np.float64)
        if free:
            self.data[tuple(idx)] = arr.reshape([self.shape[d] for d in free], order="F")
        else:
            self.data[tuple(idx)] = arr[0]
        del target


def parse_decls(path, params):
    """Parse ``real(kind=rb) :: a(dims), b(dims)`` declarations."""
    decls = {}
    text = open(path).read()
    for _, stmt in statements(text):
        m = re.match(r"(?i)^real\s*\(\s*kind\s*=\s*rb\s*\)\s*(?:,\s*dimension\s*\(([^)]*)\))?\s*::\s*(.*)$", stmt)
        if not m:
            continue
        body = m.group(2)
        # split on commas not inside parentheses
        depth = 0
        parts, cur = [], ""
        for ch in body:
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            if ch == "," and depth == 0:
                parts.append(cur)
                cur = ""
            else:
                cur += ch
        parts.append(cur)
        for p in parts:
            p = p.strip()
            mm = re.match(r"(\w+)\s*(?:\(([^)]*)\))?", p)
            name = mm.group(1).lower()
            dims = mm.group(2)
            if dims is None:
                decls[name] = []
                continue
            bounds = []
            for d in dims.split(","):
                d = d.strip().lower()
                if ":" in d:
                    lo, hi = d.split(":")
                    bounds.append((_ival(lo, params), _ival(hi, params)))
                else:
                    bounds.append((1, _ival(d, params)))
            decls[name] = bounds
    return decls


def _ival(s, params):
    s = s.strip().lower()
    if s in params:
        return params[s]
    return int(s)


def parse_assignments(path, wanted_subs, decls_for_sub, scalars_ok=True):
    """Collect array/scalar assignments inside the named subroutines."""
    arrays = {}
    text = open(path).read()
    for sub, stmt in statements(text):
        if sub not in wanted_subs:
            continue
        m = re.match(r"^(\w+)\s*(\(([^=]*)\))?\s*=\s*(.*)$", stmt)
        if not m:
            continue
        name = m.group(1).lower()
        subs = m.group(3)
        rhs = m.group(4)
        decls = decls_for_sub(sub)
        if name not in decls:
            continue
        key = (sub, name)
        if key not in arrays:
            bounds = decls[name]
            arrays[key] = FArray(bounds) if bounds else None
        if "irradscl" in rhs:
            continue  # handled explicitly (band 29 rescaling)
        vals = parse_values(rhs)
        if not decls[name]:
            arrays[key] = vals[0]
        else:
            arrays[key].assign(subs.split(","), vals)
    return arrays


def main(ref):
    src = os.path.join(ref, "src")
    mod = os.path.join(ref, "modules")

    # ---- g-point mapping, weights: rrtmg_sw_init.f90 swcmbdat ----
    init_path = os.path.join(src, "rrtmg_sw_init.f90")
    init_text = open(init_path).read()
    ints = {}
    wt = None
    for sub, stmt in statements(init_text):
        if sub != "swcmbdat":
            continue
        m = re.match(r"^(ngc|ngs|ngm|ngn|ngb)\s*\(:\)\s*=\s*\(/(.*)/\)$", stmt)
        if m:
            ints[m.group(1)] = [int(t) for t in m.group(2).split(",") if t.strip()]
        m = re.match(r"^wt\s*\(:\)\s*=\s*(.*)$", stmt)
        if m:
            wt = np.array(parse_values(m.group(1)))
    ngc, ngs, ngm, ngn, ngb = (ints[k] for k in ("ngc", "ngs", "ngm", "ngn", "ngb"))
    assert len(ngm) == 224 and len(ngn) == 112 and len(wt) == 16

    # rwgt: rrtmg_sw_init.f90:130-154
    rwgt = np.zeros(224)
    igcsm = 0
    for ibnd in range(14):
        wtsm = np.zeros(16)
        if ngc[ibnd] < 16:
            for igc in range(ngc[ibnd]):
                igcsm += 1
                wtsum = 0.0
                ipr0 = sum(ngn[ngs[ibnd] - ngc[ibnd]: ngs[ibnd] - ngc[ibnd] + igc])
                for ipr in range(ngn[igcsm - 1]):
                    wtsum = wtsum + wt[ipr0 + ipr]
                wtsm[igc] = wtsum
            for ig in range(16):
                ind = ibnd * 16 + ig
                rwgt[ind] = wt[ig] / wtsm[ngm[ind] - 1]
        else:
            for ig in range(16):
                igcsm += 1
                rwgt[ibnd * 16 + ig] = 1.0

    # ---- k-distribution data ----
    kg_path = os.path.join(src, "rrtmg_sw_k_g.f90")
    band_decls = {}
    for b in BANDS:
        params = {"no%d" % b: 16, "ng%d" % b: NG[b]}
        band_decls[b] = parse_decls(os.path.join(mod, "rrsw_kg%d.f90" % b), params)
    kg = parse_assignments(kg_path, {"sw_kgb%d" % b for b in BANDS},
                           lambda sub: band_decls[int(sub[6:])])

    # band 29 rescaling of irradnceo (rrtmg_sw_k_g.f90:62460-62461); the
    # scale factor is a default real, which the reference makefiles promote
    # to FP64 (-r8)
    irradscl = 13.221 / (13.221 - 0.455)
    kg[("sw_kgb29", "irradnceo")].data[:] = irradscl * kg[("sw_kgb29", "irradnceo")].data

    records = []

    def add(name, arr):
        a = np.asarray(arr, dtype=np.float64)
        if a.ndim == 0:
            a = a.reshape(1)
        if np.isnan(a).any():
            raise ValueError("unfilled values in " + name)
        records.append((name, a))

    # ---- reduction 224 -> 112 (cmbgb16s .. cmbgb29) ----
    for bi, b in enumerate(BANDS):
        sub = "sw_kgb%d" % b
        decl = band_decls[b]
        g0 = sum(ngn[: ngs[bi] - ngc[bi]])  # unused; kept for clarity of mapping
        del g0
        groups = []
        ipr = 0
        for igc in range(ngc[bi]):
            n = ngn[ngs[bi] - ngc[bi] + igc]
            groups.append(list(range(ipr, ipr + n)))
            ipr += n
        assert ipr == 16
        w = rwgt[bi * 16: bi * 16 + 16]
        for (s, name), val in sorted(kg.items()):
            if s != sub:
                continue
            if name.endswith("o") and decl.get(name) and name[:-1] in decl:
                arr = val.data
                # the original-g dimension is the first one for the solar
                # source arrays and rayla, the last one otherwise
                gdim = 0 if name in SOURCE_NAMES or name == "raylao" else arr.ndim - 1
                assert arr.shape[gdim] == 16, (b, name)
                weighted = name not in SOURCE_NAMES
                out_shape = list(arr.shape)
                out_shape[gdim] = ngc[bi]
                out = np.zeros(out_shape, order="F")
                for igc, grp in enumerate(groups):
                    acc = np.zeros([s_ for i_, s_ in enumerate(arr.shape) if i_ != gdim])
                    for ip in grp:
                        sl = np.take(arr, ip, axis=gdim)
                        acc = acc + (sl * w[ip] if weighted else sl)
                    idx = [slice(None)] * arr.ndim
                    idx[gdim] = igc
                    out[tuple(idx)] = acc
                add("b%d.%s" % (b, name[:-1]), out)
            elif name == "rayl" and not decl[name]:
                add("b%d.rayl" % b, np.array([val]))
    # ---- reference atmosphere: rrtmg_sw_setcoef.f90:308-362 ----
    ref_decl = {"pref": [(1, 59)], "preflog": [(1, 59)], "tref": [(1, 59)]}
    ref = parse_assignments(os.path.join(src, "rrtmg_sw_setcoef.f90"), {"swatmref"},
                            lambda sub: ref_decl)
    for name in ("pref", "preflog", "tref"):
        add(name, ref[("swatmref", name)].data)

    # ---- cloud LUTs: rrtmg_sw_init.f90 swcldpr; shapes modules/rrsw_cld.f90 ----
    cld_decl = parse_decls(os.path.join(mod, "rrsw_cld.f90"), {})
    cld = parse_assignments(init_path, {"swcldpr"}, lambda sub: cld_decl)
    for name in ("extliq1", "ssaliq1", "asyliq1", "extice2", "ssaice2", "asyice2",
                 "extice3", "ssaice3", "asyice3", "fdlice3",
                 "abari", "bbari", "cbari", "dbari", "ebari", "fbari"):
        add(name, cld[("swcldpr", name)].data)

    # ---- aerosol: swaerpr; shapes modules/rrsw_aer.f90 ----
    aer_decl = {n: [(1, 14), (1, 6)] for n in ("rsrtaua", "rsrpiza", "rsrasya")}
    aer = parse_assignments(init_path, {"swaerpr"}, lambda sub: aer_decl)
    for name in ("rsrtaua", "rsrpiza", "rsrasya"):
        add(name, aer[("swaerpr", name)].data)

    # ---- spectral band limits: swdatinit ----
    for sub, stmt in statements(init_text):
        if sub != "swdatinit":
            continue
        m = re.match(r"^(wavenum1|wavenum2)\s*\(:\)\s*=\s*(.*)$", stmt)
        if m:
            add(m.group(1), parse_values(m.group(2)))
    # ---- mean solar cycle Mg / SB index tables: rrtmg_sw_rad.f90 inatm_sw ----
    cyc_decl = {"mgavgcyc": [(1, 134)], "sbavgcyc": [(1, 134)]}
    cyc = parse_assignments(os.path.join(src, "rrtmg_sw_rad.f90"), {"inatm_sw"},
                            lambda sub: cyc_decl)
    for name in ("mgavgcyc", "sbavgcyc"):
        add(name, cyc[("inatm_sw", name)].data)
    add("ngb", np.array(ngb, dtype=np.float64))
    add("rwgt", rwgt)

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rrtmg_sw_tables.bin")
    with open(out, "wb") as f:
        f.write(b"RRSWTB01")
        f.write(struct.pack("<I", len(records)))
        for name, a in records:
            nb = name.encode()
            assert len(nb) < 32
            f.write(nb + b"\0" * (32 - len(nb)))
            dims = list(a.shape) + [1] * (4 - a.ndim)
            f.write(struct.pack("<I4IQ", a.ndim, *dims, a.size))
            f.write(a.astype("<f8").tobytes(order="F"))
    total = sum(a.size for _, a in records)
    print("wrote %s: %d records, %d values" % (out, len(records), total))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <RRTMG_SW source tree>" % sys.argv[0])
    main(sys.argv[1])
