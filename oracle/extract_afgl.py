"""Extract the six built-in model atmospheres of rrtatm.f to JSON.

TEST INFRASTRUCTURE ONLY (data for oracle/rrtatm.py).  Run once where the
RRTMG_SW source tree is present:
``python oracle/extract_afgl.py <path-to-RRTMG_SW>``; the output,
``oracle/afgl_atmospheres.json``, is committed.

The atmospheres are physics data (AFGL tropical, mid-latitude summer and
winter, sub-arctic summer and winter, U.S. standard 1976) that the profile
builder's BLOCK DATA MLATMB (rrtatm.f:1812-2918) sets: 50 altitudes (km),
and per model the pressures (mb), temperatures (K), the mixing ratios (ppmv)
of H2O, CO2, O3, N2O, CO, CH4, O2 and the total air density (cm-3).  The
arrays AMOLmk hold model m's species k; they are read here from the fixed-
form DATA statements (columns 1-72, continuation in column 6), the repeat
fill past the 50 levels ignored.
"""
import json
import os
import re
import sys


def statements(lines):
    """Fixed-form Fortran statements: comments dropped, columns 73+ cut, continuations joined."""
    out = []
    for line in lines:
        if not line or line[0] in "Cc*!":
            continue
        body = line[:72]
        if len(body) > 5 and body[5] not in " 0" and out:
            out[-1] += body[6:]
        else:
            out.append(body)
    return out


def block(lines, name):
    start = next(i for i, ln in enumerate(lines) if re.match(r"\s+BLOCK DATA %s\b" % name, ln[:72]))
    end = next(i for i in range(start + 1, len(lines)) if re.match(r"\s+END\s*$", lines[i][:72]))
    return lines[start:end]


def data_arrays(stmts):
    arrays = {}
    for st in stmts:
        m = re.match(r"\s*DATA\s+(\w+)\s*/(.*)/\s*$", st)
        if not m:
            continue
        vals = []
        for tok in m.group(2).split(","):
            tok = tok.strip()
            if not tok or "*" in tok:
                continue
            vals.append(float(tok))
        arrays[m.group(1)] = vals
    return arrays


def main(ref):
    lines = open(os.path.join(ref, "src", "rrtatm.f")).read().splitlines()
    arr = data_arrays(statements(block(lines, "MLATMB")))
    out = {
        "source": "rrtatm.f BLOCK DATA MLATMB: the six built-in model atmospheres",
        "models": ["tropical", "midlatitude summer", "midlatitude winter", "subarctic summer",
                   "subarctic winter", "U.S. standard 1976"],
        "alt": arr["ALT"][:50],
        "p": [arr["P%d" % m][:50] for m in range(1, 7)],
        "t": [arr["T%d" % m][:50] for m in range(1, 7)],
        "amol": [[arr["AMOL%d%d" % (m, k)][:50] for k in range(1, 9)] for m in range(1, 7)],
    }
    assert len(out["alt"]) == 50 and all(len(a) == 50 for m in out["amol"] for a in m)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "afgl_atmospheres.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <RRTMG_SW source tree>" % sys.argv[0])
    main(sys.argv[1])
