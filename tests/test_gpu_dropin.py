"""The drop-in stage executables (bin/int1e, int2e, scf, ao2mo, mp2) run in a
scratch directory on the reference's inputs (envdat, nucpos, fmem, mybasis,
Ftab), chained through the reference's files exactly as its driver chains its
own programs, against the oracle: integrals in the files, the printed SCF and
MP2 energies.  RHF (CO2) and UHF (O triplet)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import golden
from myqc_gb300 import formats
from myqc_gb300.build import BINDIR

pytestmark = pytest.mark.gpu


def _run(stage, cwd):
    r = subprocess.run([os.path.join(BINDIR, stage)], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (stage, r.stdout[-2000:], r.stderr[-2000:])
    assert not os.path.exists(os.path.join(cwd, "error")), (stage, r.stdout[-2000:])
    return r.stdout


def _number(pattern, text):
    m = re.search(pattern + r"\s*(-?\d+\.\d+(?:[EeDd][+-]?\d+)?)", text)
    assert m, (pattern, text[-1500:])
    return float(m.group(1).replace("D", "E"))


@pytest.mark.parametrize("name", ["CO2", "O_triplet"])
def test_stage_chain(tmp_path, ftab, basis_text, name):
    zt = open(golden("zmat", name + ".ZMAT")).read()
    sysm = formats.parse_zmat_text(zt)
    sysm.options[8] = 10  # SCF threshold 1e-10, as the oracle run below
    sysm.options[1] = 1   # MP2
    formats.write_env(sysm, str(tmp_path))
    shutil.copy(golden("mybasis"), tmp_path / "mybasis")
    shutil.copy(golden("Ftab"), tmp_path / "Ftab")
    out = "".join(_run(s, str(tmp_path)) for s in ("int1e", "int2e", "scf", "ao2mo", "mp2"))
    ref = O.run_job(zt, basis_text, ftab, 0, conv_exp=10)
    n = ref["S"].shape[0]
    S = formats.read_text_numbers(str(tmp_path / "Suv")).reshape(n, n, order="F")
    assert np.max(np.abs(S - ref["S"])) < 1e-11
    XX = np.frombuffer(formats.read_records(str(tmp_path / "XX"))[0], "<f8").reshape((n,) * 4, order="F")
    assert np.max(np.abs(XX - ref["XX"])) < 1e-10
    E = _number(r"Total SCF energy \(a\.u\)", out)
    assert abs(E - ref["scf"].energy) < 1e-9, (E, ref["scf"].energy)
    Emp2 = _number(r"E\(MBPT2\) =", out)
    mp2 = ref["mp2"] if "mp2" in ref else O.mp2(ref["mol"], ref["scf"], ref["XX"])
    assert abs(Emp2 - mp2["E_MP2"]) < 1e-8, (Emp2, mp2)
    for f in ("Cui", "eig", "MOLDEN", "ijab_AB", "basinfo", "setinfo"):
        assert (tmp_path / f).exists(), f
    # a stage started after a failure does nothing
    (tmp_path / "error").write_text("")
    r = subprocess.run([os.path.join(BINDIR, "scf")], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0 and "STARTING SCF" not in r.stdout
