"""The drop-in stage executables (bin/parse, int1e, int2e, scf, ao2mo, mp2)
run in a scratch directory on the reference's inputs (ZMAT or envdat, nucpos,
fmem; mybasis, Ftab), chained through the reference's files exactly as its
driver chains its own programs, against the oracle: integrals in the files,
the printed SCF and MP2 energies (RHF CO2, UHF O triplet), and the MOLDEN
file against the reference's own (Be, O singlet, NO)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import golden, molden_header_values, molden_orbital_errors, read_molden
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


@pytest.mark.parametrize("name,tol_e,tol_p", [("Be", 2e-8, 1e-8), ("O_singlet", 2e-8, 1e-8), ("NO", 1.5e-7, 2e-6)])
def test_molden_from_zmat(tmp_path, basis_text, name, tol_e, tol_p):
    """parse -> int1e -> int2e -> scf from the example's ZMAT alone, and the
    MOLDEN file the scf stage writes against the one the reference wrote for
    the same input: the same header up to [MO] (atoms, the mybasis sections
    in list-directed layout) -- the very text where the reference's file
    comes from a gfortran that prints 17 digits (O singlet, NO), the same
    values where it printed 15 (Be) -- then the orbitals -- energies, occupations and
    degenerate-set projectors, up to a common rotation of the p functions
    (none is fixed for an atom or a linear molecule).  The reference's
    SCF_Conv default (1e-7 on the density) bounds the NO agreement."""
    shutil.copy(golden("zmat", name + ".ZMAT"), tmp_path / "ZMAT")
    shutil.copy(golden("mybasis"), tmp_path / "mybasis")
    shutil.copy(golden("Ftab"), tmp_path / "Ftab")
    out = "".join(_run(s, str(tmp_path)) for s in ("parse", "int1e", "int2e", "scf"))
    assert "Total SCF energy" in out
    head, mos = read_molden((tmp_path / "MOLDEN").read_text())
    ref_head, ref_mos = read_molden(open(golden("molden", name + ".MOLDEN")).read())
    assert molden_header_values(head) == molden_header_values(ref_head)
    if name != "Be":
        assert head == ref_head
    sysm = formats.read_env(str(tmp_path))
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    de, occ_ok, dp = molden_orbital_errors(mos, ref_mos, basis.basinfo)
    assert de < tol_e and occ_ok and dp < tol_p, (de, occ_ok, dp)


def test_chain_from_zmat(tmp_path, ftab, basis_text):
    """The whole chain from the ZMAT of the reference's CO2 example, the way
    its driver runs it (parse first): the printed MP2 energy against the
    oracle's run of the same input."""
    zt = open(golden("zmat", "CO2.ZMAT")).read()
    (tmp_path / "ZMAT").write_text(zt)
    shutil.copy(golden("mybasis"), tmp_path / "mybasis")
    shutil.copy(golden("Ftab"), tmp_path / "Ftab")
    out = "".join(_run(s, str(tmp_path)) for s in ("parse", "int1e", "int2e", "scf", "ao2mo", "mp2"))
    ref = O.run_job(zt, basis_text, ftab, 0)
    assert abs(_number(r"Total SCF energy \(a\.u\)", out) - ref["scf"].energy) < 1e-8
    assert abs(_number(r"E\(MBPT2\) =", out) - ref["mp2"]["E_MP2"]) < 1e-7


def test_cis_blocks(tmp_path, ftab, basis_text):
    """UHF CIS integral files of the ao2mo stage (EXCITE= CIS, CALC= SCF) on the
    reference's OH example: every record of ajib_AA, ajbi_AA, ajib_AB, ajib_BB
    and ajbi_BB against the oracle's restatement of slow_ao2mo_CIS_UHF, applied
    to the XX and Cui files the earlier stages wrote (the orbitals' signs are
    the scf stage's own).  A CIS request on an RHF reference fails as the
    reference does."""
    zt = open(golden("zmat", "OH.ZMAT")).read()
    sysm = formats.parse_zmat_text(zt)
    assert sysm.options[13] == 1 and sysm.options[1] == 0 and sysm.options[3] == 1
    sysm.options[8] = 10
    formats.write_env(sysm, str(tmp_path))
    shutil.copy(golden("mybasis"), tmp_path / "mybasis")
    shutil.copy(golden("Ftab"), tmp_path / "Ftab")
    for s in ("int1e", "int2e", "scf", "ao2mo"):
        _run(s, str(tmp_path))
    XX = np.frombuffer(formats.read_records(str(tmp_path / "XX"))[0], "<f8")
    n = int(round(XX.size ** 0.25))
    XX = XX.reshape((n,) * 4, order="F")
    C = formats.read_text_numbers(str(tmp_path / "Cui"))
    CA, CB = C[:n * n].reshape(n, n, order="F"), C[n * n:2 * n * n].reshape(n, n, order="F")
    ref = O.cis_records(XX, CA, CB, sysm.nelcA, sysm.nelcB)
    for name, recs in ref.items():
        got = formats.read_records(str(tmp_path / name))
        assert len(got) == len(recs), name
        for g, r in zip(got, recs):
            g = np.frombuffer(g, "<f8")
            assert g.shape == r.shape and np.max(np.abs(g - r)) < 1e-12, name
    # RHF reference: the reference's ao2mo stops with an error
    sysm.options[3] = 0
    formats.write_env(sysm, str(tmp_path))
    r = subprocess.run([os.path.join(BINDIR, "ao2mo")], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode != 0 and (tmp_path / "error").exists()


def test_props_dipole(tmp_path, ftab, basis_text):
    """PROP= first on an SCF of HF: the props stage (int1p, then cphf) after int1e,
    int2e and scf prints the dipole moment of cphf_dipole_rhf, computed from the
    Pxuv and Da files; it matches the oracle's dipole integrals contracted with
    the oracle's SCF density (1e-8), and Pxuv matches the oracle's integrals."""
    zt = open(golden("zmat", "HF.ZMAT")).read()
    sysm = formats.parse_zmat_text(zt)
    sysm.options[8] = 10
    sysm.options[1] = 0
    sysm.options[16] = 1
    formats.write_env(sysm, str(tmp_path))
    shutil.copy(golden("mybasis"), tmp_path / "mybasis")
    shutil.copy(golden("Ftab"), tmp_path / "Ftab")
    out = "".join(_run(s, str(tmp_path)) for s in ("int1e", "int2e", "scf", "props"))
    ref = O.run_job(zt, basis_text, ftab, 0, conv_exp=10)
    mol = ref["mol"]
    P = O.int1p(mol, ref["basis"], 0)
    n = P.shape[1]
    Pf = formats.read_text_numbers(str(tmp_path / "Pxuv"))
    assert np.max(np.abs(Pf.reshape(3, n * n) - P.reshape(3, n, n).transpose(0, 2, 1).reshape(3, n * n))) < 1e-11
    mu = O.dipole_moment(P, O.density(ref["scf"].C, mol.nelcA, 2.0), mol)
    m = re.search(r"X\s+Y\s+Z\s*\n\s*(-?\d+\.\d+)\s+(-?\d+\.\d+)\s+(-?\d+\.\d+)", out)
    assert m, out[-1500:]
    got = np.array([float(g) for g in m.groups()])
    assert np.max(np.abs(got - mu)) < 2e-6, (got, mu)  # printed with 6 decimals (F15.6)
    Da = np.frombuffer(formats.read_records(str(tmp_path / "Da"))[0], "<f8").reshape(n, n, order="F")
    assert np.max(np.abs(O.dipole_moment(P, Da, mol) - mu)) < 1e-8
