"""The parse drop-in stage (src/parser/parser.f90) on the CPU: ZMAT ->
envdat, nucpos, fmem.  Its files must read back (getenv, src/myQC/env.f90)
to exactly the values of formats.parse_zmat_text, the restatement the other
tests build their systems with, on every ZMAT the reference ships; and its
error paths must leave `error` behind with a nonzero status, as the
reference's parser does (or, where that only STOPs, as a driver needs)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from myqc_gb300 import formats
from myqc_gb300.build import BINDIR

PARSE = os.path.join(BINDIR, "parse")
ZMATS = sorted(f[:-5] for f in os.listdir(os.path.join(GOLDEN, "zmat")) if f.endswith(".ZMAT"))


def _parse(tmp_path, text):
    if not os.path.exists(PARSE):
        pytest.skip("stage executables not built")
    for f in ("envdat", "nucpos", "fmem", "error"):
        if (tmp_path / f).exists():
            (tmp_path / f).unlink()
    (tmp_path / "ZMAT").write_text(text)
    return subprocess.run([PARSE], cwd=str(tmp_path), capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("name", ZMATS)
def test_parse_matches_restatement(tmp_path, name):
    text = open(os.path.join(GOLDEN, "zmat", name + ".ZMAT")).read()
    r = _parse(tmp_path, text)
    assert r.returncode == 0 and not (tmp_path / "error").exists(), r.stdout
    got = formats.read_env(str(tmp_path))
    want = formats.parse_zmat_text(text)
    assert np.array_equal(got.atoms, want.atoms)
    assert np.array_equal(got.xyz, want.xyz)  # bit for bit: same operations in the same order
    assert (got.nelcA, got.nelcB) == (want.nelcA, want.nelcB)
    assert got.options == want.options
    assert float(open(tmp_path / "fmem").read().split()[0]) == want.options[6]
    assert text.split("\n")[0] in r.stdout  # the input is echoed


def test_parse_units_and_options(tmp_path):
    text = ("CARTESIAN\nO 0.0 0.0 0.0\nH 0.0 1.43 1.1\nH 0.0 -1.43 1.1D0\nEND\n\n"
            "CALC= MP2\nBASIS= STO-3G\nUNITS= Bohr\nSCF_Conv= 10\nMEMORY= -5\nPAR= OMP\nVERB= 2\nE_NUM= -3\nBOGUS= 1\n")
    r = _parse(tmp_path, text)
    assert r.returncode == 0, r.stdout
    got = formats.read_env(str(tmp_path))
    assert got.options[11] == 1 and got.options[8] == 10 and got.options[6] == 1000
    assert got.options[4] == 2 and got.options[7] == 2 and got.options[15] == 1
    assert "could not understand" in r.stdout
    # bohr input: recentred only
    X = np.array([[0, 0, 0], [0, 1.43, 1.1], [0, -1.43, 1.1]])
    com = (16 * X[0] + X[1] + X[2]) / 18
    assert np.allclose(got.xyz, X - com, atol=1e-15)
    assert (got.nelcA, got.nelcB) == (5, 5)


@pytest.mark.parametrize("text,needle", [
    ("INTERNAL\nO\nEND\n", "not supported"),
    ("CARTESIAN\nO 0 0 0\nH 0 0 1\n", "END"),
    ("CARTESIAN\nXx 0 0 0\nEND\n", "element"),
    ("CARTESIAN\nEND\n\nCALC= SCF\n", "No atoms"),
    ("CARTESIAN\nO 0 0 0\nEND\n\nCALC= CCSD\n", "method"),
    ("CARTESIAN\nO 0 0 0\nEND\n\nREF= ROHF\n", "reference"),
    ("CARTESIAN\nO 0 0 0\nEND\n\nMULTI= 0\n", "multiplicity"),
    ("CARTESIAN\nO 0 0 0\nH 0 0 0.1\nEND\n\nREF= UHF\nMULTI= 2\n", "too close"),
    ("CARTESIAN\nO 0 0 0\nH 0 0 1\nEND\n\nREF= RHF\nMULTI= 2\n", "RHF for open shell"),
    ("CARTESIAN\nO 0 0 0\nH 0 0 1\nEND\n\nREF= UHF\nMULTI= 1\n", "not allowed"),
    ("CARTESIAN\nO 0 0 0\nEND\n\nCALC= MP2\nEXCITE= CIS\nREF= UHF\nMULTI= 3\n", "only SCF CIS"),
    ("CARTESIAN\nO 0 0 0\nEND\n\nCALC= SCF\nPROP= 1\nREF= UHF\nMULTI= 3\n", "only RHF reference"),
])
def test_parse_errors(tmp_path, text, needle):
    r = _parse(tmp_path, text)
    assert r.returncode != 0 and (tmp_path / "error").exists()
    assert needle in r.stdout, r.stdout


def test_parse_missing_zmat(tmp_path):
    if not os.path.exists(PARSE):
        pytest.skip("stage executables not built")
    r = subprocess.run([PARSE], cwd=str(tmp_path), capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and (tmp_path / "error").exists() and "ZMAT" in r.stdout
