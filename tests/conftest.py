import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmyqc.so")


def golden(*p):
    return os.path.join(GOLDEN, *p)


@pytest.fixture(scope="session")
def ftab():
    import oracle
    return oracle.read_ftab(golden("Ftab"))


@pytest.fixture(scope="session")
def basis_text():
    return open(golden("mybasis")).read()


@pytest.fixture(scope="session")
def ctx():
    from myqc_gb300.session import Context
    c = Context(0)
    yield c
    c.close()


# ---------------------------------------------------------------- MOLDEN files
def read_molden(text):
    """The lines up to and including [MO], and the orbitals as (spin, energy,
    occupation as printed, coefficients)."""
    import numpy as np
    lines = text.split("\n")
    k = next(i for i, ln in enumerate(lines) if ln.strip() == "[MO]")
    mos, i = [], k + 1
    while i < len(lines):
        if lines[i].strip().startswith("Sym="):
            ene, spin, occ = float(lines[i + 1].split()[1]), lines[i + 2].split()[1], lines[i + 3].split()[1]
            i += 4
            c = []
            while i < len(lines) and lines[i].strip() and not lines[i].strip().startswith("Sym="):
                c.append(float(lines[i].split()[1]))
                i += 1
            mos.append((spin, ene, occ, np.array(c)))
        else:
            i += 1
    return lines[:k + 1], mos


def molden_header_values(lines):
    """The header of a MOLDEN file (read_molden's first part) as tokens, the
    numbers as floats: compares files written by gfortran versions whose
    list-directed REAL(8) items print 15 or 17 digits and blank lines with or
    without a space."""
    out = []
    for ln in lines:
        for t in ln.split():
            try:
                out.append(float(t.replace("D", "E")))
            except ValueError:
                out.append(t)
    return out


def molden_orbital_errors(mos, ref_mos, basinfo, degenerate=1e-5):
    """How far the orbitals `mos` are from `ref_mos` (both as read_molden
    returns them), invariant to what a MOLDEN file does not fix: the sign of
    each orbital, rotations inside a set of degenerate orbitals, and a common
    rotation of every atom's p functions (an atom or a linear molecule has no
    preferred orientation around its axis).  The rotation is taken from the
    eigenvectors of the two files' p-block occupied densities (the 3 x 3
    blocks summed over atoms, beta weighted by one half), with the signs of
    the axes chosen to match the densities best.  Returns the largest energy
    difference, whether every occupation string agrees, and the largest
    difference of the projectors onto each set of degenerate orbitals (energies
    of the reference within `degenerate`)."""
    import itertools

    import numpy as np
    bi = np.asarray(basinfo)[2:].reshape(-1, 5)
    n = len(ref_mos[0][3])
    px = [o for o in range(n) if bi[o, 1] == 1 and bi[o, 2] == 0]

    def by_spin(ms):
        return {sp: [m for m in ms if m[0] == sp] for sp in ("Alpha", "Beta")}

    A, B = by_spin(mos), by_spin(ref_mos)

    def pblock(ms):
        M = np.zeros((3, 3))
        for w, sp in ((1.0, "Alpha"), (0.5, "Beta")):
            for m in ms[sp]:
                if float(m[2]) > 0:
                    for o in px:
                        v = m[3][o:o + 3]
                        M += w * np.outer(v, v)
        return M

    def rotate(R, c):
        c = c.copy()
        for o in px:
            c[o:o + 3] = R @ c[o:o + 3]
        return c

    def dens(ms, R=None):
        out = []
        for sp in ("Alpha", "Beta"):
            D = np.zeros((n, n))
            for m in ms[sp]:
                if float(m[2]) > 0:
                    c = m[3] if R is None else rotate(R, m[3])
                    D += np.outer(c, c)
            out.append(D)
        return out

    _, V = np.linalg.eigh(pblock(A))
    _, Vr = np.linalg.eigh(pblock(B))
    Dr = dens(B)
    best = None
    for sg in itertools.product((1.0, -1.0), repeat=3):
        R = Vr @ np.diag(sg) @ V.T
        err = max(float(np.max(np.abs(x - y))) for x, y in zip(dens(A, R), Dr))
        if best is None or err < best[0]:
            best = (err, R)
    R = best[1]
    de, occ_ok, dp = 0.0, True, 0.0
    for sp in ("Alpha", "Beta"):
        a, b = A[sp], B[sp]
        assert len(a) == len(b), (sp, len(a), len(b))
        if not b:
            continue
        de = max(de, max(abs(x[1] - y[1]) for x, y in zip(a, b)))
        occ_ok = occ_ok and all(x[2] == y[2] for x, y in zip(a, b))
        i = 0
        while i < len(b):
            j = i + 1
            while j < len(b) and abs(b[j][1] - b[i][1]) < degenerate:
                j += 1
            P = sum(np.outer(rotate(R, a[k][3]), rotate(R, a[k][3])) for k in range(i, j))
            Pr = sum(np.outer(b[k][3], b[k][3]) for k in range(i, j))
            dp = max(dp, float(np.max(np.abs(P - Pr))))
            i = j
    return de, occ_ok, dp


def molden_text_of(mol, eig, C, uhf):
    """The orbital section of a MOLDEN file from energies and coefficients
    (column per orbital), in the scf stage's layout: for comparing the oracle's
    orbitals with read_molden's view of a file."""
    out = [" [MO]"]
    eigs = [eig[0], eig[1]] if uhf else [eig]
    Cs = [C[0], C[1]] if uhf else [C]
    for s, (e, c) in enumerate(zip(eigs, Cs)):
        for i in range(len(e)):
            out += [" Sym= A", f" Ene= {e[i]:15.8f}", "  Spin= " + ("Beta" if s else "Alpha"),
                    " Occup= " + ("1.0" if e[i] < 0 else "0.0")]
            out += [f" {k + 1:4d}    {c[k, i]:15.10f}" for k in range(c.shape[0])]
    return "\n".join(out) + "\n"
