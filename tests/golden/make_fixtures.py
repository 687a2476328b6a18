"""Regenerate the golden fixtures in this folder from a checkout of the reference.

    python tests/golden/make_fixtures.py /path/to/myQC

Copies the reference's input data (``src/Ftab``, ``src/mybasis``, the example
ZMAT files) and extracts its known answers into ``reference_pins.json``:

* myQC's own MOLDEN orbital energies (examples/Be, examples/O/singlet,
  examples/NO) -- the reference's parity pins -- and the three MOLDEN files
  themselves (molden/), the layout the scf stage's MOLDEN writer follows;
* the CFOUR energies shipped beside some examples (examples/*/cfour/out) --
  sanity pins only, since CFOUR uses true pi, exact Boys values and
  renormalised contractions.

Nothing at run time reads the reference; the tests read only this folder.
"""
from __future__ import annotations

import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
EXAMPLES = ["Be", "O/singlet", "O/triplet", "NO", "CO2", "CO", "HeH", "OH", "H2", "HF", "H"]


def molden_energies(path):
    alpha, beta = [], []
    spin = None
    vals = []
    for ln in open(path):
        s = ln.strip()
        if s.startswith("Ene="):
            vals.append(float(s.split()[1]))
        elif s.startswith("Spin="):
            spin = s.split()[1]
            (alpha if spin == "Alpha" else beta).append(vals[-1])
    return alpha, beta


def cfour_values(path):
    txt = open(path).read()
    out = {}
    m = re.findall(r"E\(SCF\)=\s+(-?\d+\.\d+)", txt)
    if m:
        out["E_SCF"] = float(m[-1])
    for key in ("E2(AA)", "E2(AB)", "E2(TOT)"):
        mm = re.findall(re.escape(key) + r"\s*=\s*(-?\d+\.\d+)", txt)
        if mm:
            out[key] = float(mm[-1])
    return out


def main(ref):
    shutil.copyfile(os.path.join(ref, "src", "Ftab"), os.path.join(HERE, "Ftab"))
    shutil.copyfile(os.path.join(ref, "src", "mybasis"), os.path.join(HERE, "mybasis"))
    os.makedirs(os.path.join(HERE, "zmat"), exist_ok=True)
    for ex in EXAMPLES:
        shutil.copyfile(os.path.join(ref, "examples", ex, "ZMAT"),
                        os.path.join(HERE, "zmat", ex.replace("/", "_") + ".ZMAT"))
    pins = {"molden": {}, "cfour": {}}
    os.makedirs(os.path.join(HERE, "molden"), exist_ok=True)
    for ex in ("Be", "O/singlet", "NO"):
        shutil.copyfile(os.path.join(ref, "examples", ex, "MOLDEN"),
                        os.path.join(HERE, "molden", ex.replace("/", "_") + ".MOLDEN"))
        a, b = molden_energies(os.path.join(ref, "examples", ex, "MOLDEN"))
        pins["molden"][ex.replace("/", "_")] = {"alpha": a, "beta": b}
    for ex in ("CO2", "HeH", "OH"):
        pins["cfour"][ex] = cfour_values(os.path.join(ref, "examples", ex, "cfour", "out"))
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)
    print(json.dumps(pins, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_fixtures.py <path of the jhthorpe/myQC checkout>")
    main(sys.argv[1])
