"""Extract the Duan-Rokhlin known-answer output published with the reference.

    python tests/golden/make_dr_kat.py path/to/HSSC_DirectSolver

The reference's INSTALL.txt (lines 95-115) lists the indata.txt / outdata.txt pair of
its Fortran weight program (Common/FORTRAN_get_DR_weights.f): h, the wavenumber and
corr0..corr5.  This script parses those lines and writes dr_weights_kat.json beside it.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse(text: str) -> dict:
    num = r"([-+]?\d*\.\d+(?:[eEdD][-+]?\d+)?)"
    out = {}
    m = re.search(r"real_rk\s*=\s*" + num, text)
    out["k_re"] = float(m.group(1).replace("D", "e"))
    m = re.search(r"imag_rk\s*=\s*" + num, text)
    out["k_im"] = float(m.group(1).replace("D", "e"))
    m = re.search(r"^\s*h\s+=\s*" + num, text, flags=re.M)
    out["h"] = float(m.group(1).replace("D", "e"))
    for i in range(6):
        m = re.search(rf"corr{i}\s*=\s*{num}\s+{num}", text)
        out[f"corr{i}"] = [float(m.group(1).replace("D", "e")), float(m.group(2).replace("D", "e"))]
    return out


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_dr_kat.py <HSSC_DirectSolver source directory (the one holding INSTALL.txt)>")
    ref = sys.argv[1]
    kat = parse(open(os.path.join(ref, "INSTALL.txt")).read())
    kat["source"] = "HSSC_DirectSolver/INSTALL.txt:95-115 (outdata.txt of FORTRAN_get_DR_weights)"
    with open(os.path.join(HERE, "dr_weights_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    print(kat)
