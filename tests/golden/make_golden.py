"""Generate the golden fixtures of this directory from the reference sources.

Reads, as text, the constants the reference itself prints or hard-codes:
  * gll_ref.json  <- src/models/flat_shell/flat_shell_engine/gll.m:8-34
                     (GLL nodes/weights table, n = 2..10)
  * c3d_ref.json  <- src/models/common/engineering_2_C3D.m:1-24,42-51
                     (glass-epoxy engineering constants and the 3D stiffness
                     the reference prints in its comment, 1e10 Pa units)
  * homog_ref.json <- src/models/common/Homogenized_Cmatrix.m:1-7,27-37,54-58
                     (fibre/matrix inputs, the printed shell q rows and the
                     printed 3D stiffness row, 1e11 Pa units)
  * damage_ref.json <- src/models/common/damage_model.m:10-16
                     (the example 6x6 stiffness and damage degree in its comment)
Run from the repository root:  python tests/golden/make_golden.py REF_ROOT
where REF_ROOT is the reference checkout.  The fixtures are committed; the
tests never read the reference tree.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_gll(path):
    txt = open(path).read()
    out = {}
    for m in re.finditer(r"case\s+(\d+)\s*;?(.*?)(?=case|%otherwise|end;?\s*$)", txt, re.S):
        n = int(m.group(1))
        body = m.group(2)
        ksi = [None] * n
        wi = [None] * n
        for name, arr in (("ksi", ksi), ("wi", wi)):
            for a in re.finditer(name + r"\((\d+)\)\s*=\s*([^;]+);", body):
                k = int(a.group(1)) - 1
                expr = a.group(2).strip()
                arr[k] = expr
        # resolve symmetric references like -ksi(4) or wi(5)
        def val(arr, e, other):
            e = e.strip()
            neg = e.startswith("-")
            e2 = e[1:] if neg else e
            mm = re.fullmatch(r"(ksi|wi)\((\d+)\)", e2)
            if mm:
                src = arr if mm.group(1) == name_of(arr) else other
                v = val(src, src[int(mm.group(2)) - 1], arr)
            else:
                v = float(e2)
            return -v if neg else v
        def name_of(arr):
            return "ksi" if arr is ksi else "wi"
        if n >= 2 and all(x is not None for x in ksi + wi):
            out[n] = {"ksi": [val(ksi, e, wi) for e in ksi], "wi": [val(wi, e, ksi) for e in wi]}
    return out


def parse_c3d(path):
    txt = open(path).read()
    consts = {}
    for name in ("e11", "e22", "ni12", "ni23", "g12"):
        m = re.search(r"^\s*" + name + r"\s*=\s*([0-9.eE+-]+)\s*;", txt, re.M)
        consts[name] = float(m.group(1))
    block = txt[txt.index("% C ="):]
    rows = []
    for line in block.splitlines()[1:]:
        nums = re.findall(r"[-+]?\d+\.\d+|\b0\b", line)
        if len(nums) == 6:
            rows.append([float(x) for x in nums])
        if len(rows) == 6:
            break
    scale = 1e10 if "1.0e+10" in block[:200] else 1.0
    return {"inputs": consts, "C_printed": rows, "scale": scale, "digits": 4}


NUM = r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?"


def parse_homogenized(path):
    """Inputs (lines 1-7), the two printed shell rows [q11 q12 q22 q44 q55 q66]
    and the printed 3D row [q11 q12 q13 q22 q23 q33 q44 q55 q66], all in
    units of 1e11 Pa, and the printed density."""
    txt = open(path).read()
    inputs = {}
    for name in ("rhom", "rhof", "em", "ef", "nim", "nif", "vol"):
        m = re.search(r"^\s*" + name + r"\s*=\s*([0-9.eE+-]+)\s*;", txt, re.M)
        inputs[name] = float(m.group(1))
    lines = txt.splitlines()
    i2 = next(i for i, ln in enumerate(lines) if ln.strip().startswith("[q11 q12 q22"))
    i3 = next(i for i, ln in enumerate(lines) if ln.strip().startswith("[q11 q12 q13"))
    shell_rows = []
    for ln in lines[i2 + 1:i3]:
        if ln.lstrip().startswith("%") and "=" not in ln:
            nums = re.findall(NUM, ln)
            if len(nums) == 6:
                shell_rows.append([float(x) for x in nums])
    rho = float(re.search(r"%\s*rho\s*=\s*(" + NUM + ")", txt).group(1))
    solid = []
    for ln in lines[i3 + 1:]:
        if not ln.lstrip().startswith("%"):
            break
        if "1.0e+11" in ln:
            continue
        solid += [float(x) for x in re.findall(NUM, ln)]
        if len(solid) >= 9:
            break
    return {"inputs": inputs, "shell_rows": shell_rows, "solid_row": solid[:9], "rho_printed": rho,
            "scale": 1e11, "digits": 4}


def parse_damage(path):
    """The example stiffness C (6x6) and damage_degree of the comment block."""
    txt = open(path).read()
    d = float(re.search(r"%\s*damage_degree\s*=\s*([0-9.]+)\s*;", txt).group(1))
    block = txt[txt.index("% C=["):]
    rows = []
    for ln in block.splitlines():
        nums = re.findall(r"\d+\.\d+|\b0\b", ln)
        if len(nums) == 6:
            rows.append([float(x) for x in nums])
        if len(rows) == 6:
            break
    return {"damage_degree": d, "C": rows}


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: python tests/golden/make_golden.py REF_ROOT")
    ref = sys.argv[1]
    g = parse_gll(os.path.join(ref, "src/models/flat_shell/flat_shell_engine/gll.m"))
    with open(os.path.join(HERE, "gll_ref.json"), "w") as f:
        json.dump({"source": "src/models/flat_shell/flat_shell_engine/gll.m:8-34",
                   "table": {str(k): v for k, v in sorted(g.items())}}, f, indent=1)
    c = parse_c3d(os.path.join(ref, "src/models/common/engineering_2_C3D.m"))
    c["source"] = "src/models/common/engineering_2_C3D.m:5-24,42-51"
    with open(os.path.join(HERE, "c3d_ref.json"), "w") as f:
        json.dump(c, f, indent=1)
    h = parse_homogenized(os.path.join(ref, "src/models/common/Homogenized_Cmatrix.m"))
    h["source"] = "src/models/common/Homogenized_Cmatrix.m:1-7,27-37,54-58"
    with open(os.path.join(HERE, "homog_ref.json"), "w") as f:
        json.dump(h, f, indent=1)
    dm = parse_damage(os.path.join(ref, "src/models/common/damage_model.m"))
    dm["source"] = "src/models/common/damage_model.m:10-16"
    with open(os.path.join(HERE, "damage_ref.json"), "w") as f:
        json.dump(dm, f, indent=1)
    print("wrote", sorted(g), "c3d_ref.json, homog_ref.json, damage_ref.json")


if __name__ == "__main__":
    main()
