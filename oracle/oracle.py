"""CPU oracle for myQC's HF/MP2 hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module; the product (``myqc_gb300`` and ``libmyqc``) never does.

It restates the reference (jhthorpe/myQC, Fortran 90) host logic in Python and
drives the C restatement in ``oracle.c`` through ctypes:

* ``parse_zmat``    -- src/parser/parser.f90:435-547 (build), :622-678
                       (cartesian), :683-735 (read_options)
* ``parse_mybasis`` -- src/myQC/basis.f90:23-226 (buildBasis)
* ``read_ftab``     -- src/integrals/int2e.f90:160-163 (one unformatted record)
* ``scf``           -- src/scf/scf.f90:61-216 (RHF), :221-404 (UHF), RHFiter
                       :720-904, UHFiter :909-1117, getEnr :1122-1152,
                       checkConv :1157-1267, with LAPACK DSYGV taken from
                       scipy (itype=1, 'V', 'L').
* ``mp2``           -- src/ao2mo/ao2mo.f90:465-602/614-904 then
                       src/mp2/mp2.f90:79-232.

Two Boys/pi modes: ``mode=0`` restates the reference exactly ("oracle A"),
``mode=1`` is the tight FP64 oracle ("oracle B": true pi, Boys to ~1e-15).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.so")

A2B = 1.8897161646320724  # parser.f90:14
ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne"]
DEFAULT_OPTIONS = [0, 0, 0, 0, 0, 1, 1000, 1, 7, 0, 1, 0, 1, 0, 0, 0, 0]  # parser.f90:60
# checkConv's lim(0:11) (scf.f90:1177-1188).  SCF_Conv=12 (examples/CO2/ZMAT)
# indexes past the end of that array; this restatement extends the table
# with 1e-12 for it.
CONV_LIMITS = [10.0 ** (-k) for k in range(0, 13)]


def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so (gcc, -ffp-contract=off)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        c_int, c_double = ctypes.c_int, ctypes.c_double
        L.orc_boys.argtypes = [c_int, c_double, c_int, dp, dp]
        L.orc_int2e.argtypes = [c_int, c_int, c_int, c_int, dp, dp, ip, ip, c_int, dp, dp, c_int, dp]
        L.orc_int1e.argtypes = [c_int, c_int, c_int, c_int, dp, dp, ip, ip, c_int, ip, dp, dp, c_int, dp, dp]
        L.orc_int1p.argtypes = [c_int, c_int, c_int, c_int, dp, dp, ip, ip, c_int, ip, dp, c_int, dp]
        L.orc_density.argtypes = [c_int, c_int, dp, c_double, dp]
        L.orc_fock_rhf.argtypes = [c_int, dp, dp, dp]
        L.orc_fock_uhf.argtypes = [c_int, dp, dp, dp, dp, dp]
        L.orc_ao2mo.argtypes = [c_int, dp, dp, c_int, dp, c_int, dp, c_int, dp, c_int, dp]
        L.orc_mp2_rhf.argtypes = [c_int, c_int, dp, dp, dp]
        L.orc_mp2_uhf.argtypes = [c_int, c_int, c_int, c_int, dp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# file formats
def read_ftab(path: str) -> np.ndarray:
    """Ftab: one gfortran sequential record of Ft(0:120,0:22), column-major.
    Returned as a flat float64 array of 121*23 values, T fastest."""
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:4], "<i4")[0])
    if n != 121 * 23 * 8 or len(raw) != n + 8:
        raise ValueError(f"Ftab: unexpected record length {n}")
    return np.frombuffer(raw[4 : 4 + n], "<f8").copy()


# --------------------------------------------------------------------------
@dataclass
class Molecule:
    atoms: np.ndarray            # Z, int32
    xyz: np.ndarray              # bohr, shape (nnuc, 3)
    nelcA: int
    nelcB: int
    options: list = field(default_factory=lambda: list(DEFAULT_OPTIONS))


def _int_field(tok: str) -> int:
    # READ(chr,'(I8)'): the first 8 columns as an integer, blanks ignored
    s = tok[:8].strip()
    return int(s) if s else 0


def parse_zmat_text(text: str) -> Molecule:
    """Restates parser.f90 for CARTESIAN input (the only style it supports)."""
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines = lines[:-1]
    fline = len(lines)
    opts = list(DEFAULT_OPTIONS)
    if lines[0].split()[0] != "CARTESIAN":
        raise ValueError("only CARTESIAN input is supported")
    atoms, xyz = [], []
    i = 1
    while True:
        if i >= fline:
            raise ValueError("You need to put 'END' marker in ZMAT")
        tok = lines[i].split()
        if tok and tok[0] == "END":
            break
        atoms.append(ELEMENTS.index(tok[0]) + 1)
        xyz.append([float(t.replace("D", "E").replace("d", "e")) for t in tok[1:4]])
        i += 1
    nline = 1 + len(atoms) + 1
    rline = fline - nline - 1
    keys = {"CALC=": 1, "BASIS=": 2, "CHARGE=": 9, "MULTI=": 10, "REF=": 3, "PAR=": 4, "NODES=": 5,
            "MEMORY=": 6, "VERB=": 7, "SCF_Conv=": 8, "UNITS=": 11, "AO2MO=": 12, "EXCITE=": 13,
            "ROOT_ALG=": 14, "E_NUM=": 15, "PROP=": 16}
    for ln in lines[nline + 1 : nline + 1 + rline]:
        tok = ln.split()
        if len(tok) < 2 or tok[0] not in keys:
            continue
        k, v = tok[0], tok[1]
        idx = keys[k]
        if k == "CALC=":
            opts[1] = {"SCF": 0, "HF": 0, "MP2": 1, "CIS": 2}[v]
        elif k == "BASIS=":
            opts[2] = {"STO-3G": 0, "tester1": 1, "tester2": 2, "tester3": 3}[v]
        elif k == "REF=":
            if v not in ("RHF", "UHF"):
                raise ValueError("bad ref")
            opts[3] = 0 if v == "RHF" else 1
        elif k == "PAR=":
            opts[4] = {"OMP": 2, "MPI": 3}.get(v, 1)
        elif k == "NODES=":
            opts[5] = 1
        elif k == "VERB=":
            opts[7] = {"1": 1, "2": 2, "3": 3}.get(v, 0)
        elif k == "UNITS=":
            opts[11] = 1 if v == "Bohr" else 0
        elif k == "AO2MO=":
            opts[12] = 1
        elif k == "EXCITE=":
            opts[13] = 1 if v in ("CIS", "1") else 0
        elif k in ("ROOT_ALG=",):
            opts[14] = 0
        elif k == "PROP=":
            opts[16] = {"NONE": 0, "ZERO": 0, "0": 0, "FIRST": 1, "1": 1, "SECOND": 2, "2": 2}.get(v, 0)
        elif k == "MEMORY=":
            val = _int_field(v)
            opts[6] = 1000 if val < 0 else val
        elif k == "E_NUM=":
            val = _int_field(v)
            opts[15] = 1 if val < 0 else val
        else:  # CHARGE= MULTI= SCF_Conv=
            opts[idx] = _int_field(v)
    atoms = np.array(atoms, dtype=np.int32)
    xyz = np.array(xyz, dtype=np.float64)
    # build(), parser.f90:435-547: centre of mass with integer masses (the
    # reference's accumulator `temp` is uninitialised; restated as 0), then
    # Angstrom -> bohr.
    mass = np.array([1.0, 4.0, 7.0, 9.0, 11.0, 12.0, 14.0, 16.0, 19.0, 20.0])
    m = mass[atoms - 1]
    com = np.zeros(3)
    temp = 0.0
    for a in range(len(atoms)):
        com = com + m[a] * xyz[a]
        temp = temp + m[a]
    com = com / temp
    xyz = xyz - com
    if opts[11] == 0:
        xyz = xyz * A2B
    charge, unpr = opts[9], opts[10] - 1
    nelc = int(atoms.sum()) - charge
    nelcA = int((nelc - unpr) / 2)
    nelcB = int((nelc - unpr) / 2)
    nelcA += unpr
    return Molecule(atoms=atoms, xyz=xyz, nelcA=nelcA, nelcB=nelcB, options=opts)


def parse_zmat(path: str) -> Molecule:
    return parse_zmat_text(open(path).read())


@dataclass
class Basis:
    bas: np.ndarray      # float64, coefficient per (set, slot)
    set: np.ndarray      # float64, exponent per set
    basinfo: np.ndarray  # int32
    setinfo: np.ndarray  # int32
    maxN: int
    maxL: int

    @property
    def ops(self) -> int:
        return int(self.basinfo[0])

    @property
    def norb(self) -> int:
        return int(self.basinfo[1])

    @property
    def nset(self) -> int:
        return int(self.setinfo[0])

    @property
    def setl(self) -> int:
        return int(self.setinfo[1])


def parse_mybasis_text(text: str, atoms, key: str = "STO-3G") -> Basis:
    """Restates buildBasis (basis.f90:23-226): the flat bas/set/basinfo/setinfo
    arrays with the reference's layout and sizes."""
    recs = [ln.split() for ln in text.split("\n")]
    first = [(r[0][:8] if r else "") for r in recs]

    def nums(r):
        return [float(t.replace("D", "E").replace("d", "e")) for t in r]

    pos = 0
    while first[pos] != key:
        pos += 1
    Smax, Cmax, Omax, almax, OpS = (int(x) for x in recs[pos + 1][:5])
    maxN, maxL = (int(x) for x in recs[pos + 2][:2])
    anum = len(atoms)
    bas = np.zeros(anum * almax * OpS)
    sets = np.zeros(anum * almax)
    basinfo = np.zeros(2 + 5 * Omax * anum, dtype=np.int32)
    setl = 3 + OpS
    setinfo = np.zeros(2 + anum * almax * setl, dtype=np.int32)
    setnum = 0
    orbnum = 0
    for i, Z in enumerate(atoms):
        name = ELEMENTS[int(Z) - 1]
        p = 0
        while first[p] != key:
            p += 1
        while first[p] != name:
            p += 1
        sec, orb, nset = (int(x) for x in recs[p + 1][:3])
        p += 2
        basinfo[0] = OpS
        basinfo[1] += orb
        setinfo[0] += nset
        setinfo[1] = setl
        for _ in range(sec):
            func, coef, pri, ang, ori = (int(x) for x in recs[p][:5])
            p += 1
            for _k in range(func):
                v = nums(recs[p][: coef + 1])
                p += 1
                val, temp = v[:coef], v[coef]
                setn = int(np.floor(abs(temp) + 0.5)) * (1 if temp >= 0 else -1)  # NINT
                sidx = setnum + setn
                sets[sidx] = val[coef - 1]
                base = 1 + sidx * setl
                setorbs = int(setinfo[base + 1])
                setinfo[base + 3] = i
                if ori == -1:
                    setinfo[base + 4 + setorbs] = orbnum
                    bas[setorbs + sidx * OpS] = val[0]
                    setorbs += 1
                elif ori == 2:
                    for m in range(3):
                        setinfo[base + 4 + setorbs] = orbnum + m
                        bas[setorbs + sidx * OpS] = val[0]
                        setorbs += 1
                    if setinfo[base + 2] < 1:
                        setinfo[base + 2] = 1
                else:
                    raise ValueError("bad angular quantum number")
                setinfo[base + 1] = setorbs
            if ori == -1:
                basinfo[2 + 5 * orbnum : 2 + 5 * (orbnum + 1)] = [pri, ang, ori, func, i]
                orbnum += 1
            else:
                for m in range(3):
                    basinfo[2 + 5 * (orbnum + m) : 2 + 5 * (orbnum + m + 1)] = [pri, ang, m, func, i]
                orbnum += 3
        setnum = int(setinfo[0])
    return Basis(bas=bas, set=sets, basinfo=basinfo, setinfo=setinfo, maxN=maxN, maxL=maxL)


def parse_mybasis(path: str, atoms) -> Basis:
    return parse_mybasis_text(open(path).read(), atoms)


# --------------------------------------------------------------------------
# integrals and digestion through the C restatement
def _xyz_colmajor(mol: Molecule) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(mol.xyz, dtype=np.float64).T).reshape(-1)


def boys(T: float, Q: int, ftab: np.ndarray, mode: int = 0) -> np.ndarray:
    out = np.zeros(Q + 1)
    rc = lib().orc_boys(mode, float(T), int(Q), np.ascontiguousarray(ftab, dtype=np.float64), out)
    if rc != 0:
        raise ValueError("Boys: Q > 16")
    return out


def int2e(mol: Molecule, basis: Basis, ftab: np.ndarray, mode: int = 0) -> np.ndarray:
    """Full XX(i,j,g,h) as an (n,n,n,n) array indexed XX[i,j,g,h]."""
    n = basis.norb
    XX = np.zeros(n ** 4)
    rc = lib().orc_int2e(basis.nset, basis.setl, basis.ops, n, basis.bas, basis.set, basis.basinfo,
                         basis.setinfo, len(mol.atoms), _xyz_colmajor(mol),
                         np.ascontiguousarray(ftab, dtype=np.float64), mode, XX)
    if rc != 0:
        raise RuntimeError("int2e failed")
    return XX.reshape(n, n, n, n, order="F")


def int1e(mol: Molecule, basis: Basis, ftab: np.ndarray, mode: int = 0):
    n = basis.norb
    S = np.zeros(n * n)
    H = np.zeros(n * n)
    rc = lib().orc_int1e(basis.nset, basis.setl, basis.ops, n, basis.bas, basis.set, basis.basinfo,
                         basis.setinfo, len(mol.atoms), np.ascontiguousarray(mol.atoms, dtype=np.int32),
                         _xyz_colmajor(mol), np.ascontiguousarray(ftab, dtype=np.float64), mode, S, H)
    if rc != 0:
        raise RuntimeError("int1e failed")
    return S.reshape(n, n, order="F"), H.reshape(n, n, order="F")


def int1p(mol: Molecule, basis: Basis, mode: int = 0) -> np.ndarray:
    """Dipole integrals Px[c] = <u| r_c |v>, c = x, y, z (int1p.f90 proc1p), (3, n, n)."""
    n = basis.norb
    Px = np.zeros(3 * n * n)
    rc = lib().orc_int1p(basis.nset, basis.setl, basis.ops, n, basis.bas, basis.set, basis.basinfo,
                         basis.setinfo, len(mol.atoms), np.ascontiguousarray(mol.atoms, dtype=np.int32),
                         _xyz_colmajor(mol), mode, Px)
    if rc != 0:
        raise RuntimeError("int1p failed")
    return np.stack([Px[c * n * n:(c + 1) * n * n].reshape(n, n, order="F") for c in range(3)])


def dipole_moment(Px: np.ndarray, D: np.ndarray, mol: Molecule) -> np.ndarray:
    """cphf_dipole_rhf (src/props/cphf.f90:80-131): mu_c = -sum_uv D(u,v) Px(c,v,u)
    + sum_A Z_A R_A,c, with D the total density (Da) and R in bohr."""
    mu = -np.einsum("uv,cvu->c", D, Px)
    xyz = np.asarray(mol.xyz, dtype=float).reshape(len(mol.atoms), 3)
    return mu + np.einsum("a,ac->c", np.asarray(mol.atoms, dtype=float), xyz)


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))


def density(C: np.ndarray, nocc: int, factor: float) -> np.ndarray:
    n = C.shape[0]
    D = np.zeros(n * n)
    lib().orc_density(n, int(nocc), _f(C), float(factor), D)
    return D.reshape(n, n, order="F")


def fock_rhf(XX: np.ndarray, D: np.ndarray) -> np.ndarray:
    n = D.shape[0]
    G = np.zeros(n * n)
    lib().orc_fock_rhf(n, _f(XX), _f(D), G)
    return G.reshape(n, n, order="F")


def fock_uhf(XX: np.ndarray, Da: np.ndarray, Db: np.ndarray):
    n = Da.shape[0]
    Ga, Gb = np.zeros(n * n), np.zeros(n * n)
    lib().orc_fock_uhf(n, _f(XX), _f(Da), _f(Db), Ga, Gb)
    return Ga.reshape(n, n, order="F"), Gb.reshape(n, n, order="F")


def nuclear_repulsion(mol: Molecule) -> float:
    """getEnr, scf.f90:1122-1152."""
    x, Z = mol.xyz, mol.atoms
    E = 0.0
    for A in range(len(Z)):
        for B in range(A):
            r = np.sqrt((x[A, 0] - x[B, 0]) ** 2 + (x[A, 1] - x[B, 1]) ** 2 + (x[A, 2] - x[B, 2]) ** 2)
            E = E + Z[A] * Z[B] / r
    return float(E)


def dsygv(A: np.ndarray, B: np.ndarray):
    """DSYGV(1,'V','L') as the reference calls it (lower triangles only)."""
    from scipy.linalg import lapack
    w, v, info = lapack.dsygv(np.tril(A), np.tril(B), itype=1, jobz="V", uplo="L")
    if info > A.shape[0]:
        raise RuntimeError("DSYGV: overlap not positive definite")
    return w, v


@dataclass
class SCFResult:
    energy: float
    eig: np.ndarray            # (n,) or (2, n)
    C: np.ndarray              # (n, n) or (2, n, n)
    D: np.ndarray              # last input density (total for RHF; (2,n,n) for UHF)
    iterations: int
    converged: bool
    enuc: float
    history: list


def scf(mol: Molecule, S: np.ndarray, H: np.ndarray, XX: np.ndarray, conv_exp: int | None = None,
        max_iter: int | None = None) -> SCFResult:
    """Plain Roothaan SCF from the core-Hamiltonian guess (scf.f90)."""
    uhf = mol.options[3] == 1
    k = mol.options[8] if conv_exp is None else conv_exp
    lim = CONV_LIMITS[k]
    Enr = nuclear_repulsion(mol)
    w, C0 = dsygv(H, S)
    hist = []
    if not uhf:
        nocc = (mol.nelcA + mol.nelcB) // 2
        cap = 500 if max_iter is None else max_iter
        C = C0
        D = density(C, nocc, 2.0)
        G = fock_rhf(XX, D)
        it, conv, eig, E = 0, False, w, 0.0
        Din = D
        while not conv:
            F = H + G
            E = 0.5 * float(np.sum(D * (F + H))) + Enr
            eig, C = dsygv(F, S)
            Din = D
            D = density(C, nocc, 2.0)
            G = fock_rhf(XX, D)
            mdiff = float(np.max(np.abs(Din - D))) if it > 0 else float("nan")
            hist.append((E, mdiff))
            if it > 0:
                conv = mdiff < lim
            it += 1
            if it >= cap:
                break
        return SCFResult(E, eig, C, Din, it, conv, Enr, hist)
    cap = 300 if max_iter is None else max_iter
    CA, CB = C0.copy(), C0.copy()
    Da = density(CA, mol.nelcA, 1.0)
    Db = density(CB, mol.nelcB, 1.0)
    Ga, Gb = fock_uhf(XX, Da, Db)
    it, conv = 0, False
    E, eA, eB = 0.0, w, w
    Dain, Dbin = Da, Db
    while not conv:
        FA, FB = H + Ga, H + Gb
        E = 0.5 * float(np.sum(Da * (FA + H) + Db * (FB + H))) + Enr
        eA, CA = dsygv(FA, S)
        eB, CB = dsygv(FB, S)
        Dain, Dbin = Da, Db
        Da = density(CA, mol.nelcA, 1.0)
        Db = density(CB, mol.nelcB, 1.0)
        Ga, Gb = fock_uhf(XX, Da, Db)
        mdiff = max(float(np.max(np.abs(Dain - Da))), float(np.max(np.abs(Dbin - Db)))) if it > 0 else float("nan")
        hist.append((E, mdiff))
        if it > 0:
            conv = mdiff < lim
        it += 1
        if it >= cap:
            break
    return SCFResult(E, np.stack([eA, eB]), np.stack([CA, CB]), np.stack([Dain, Dbin]), it, conv, Enr, hist)


def ao2mo(XX: np.ndarray, Ci, Ca, Cj, Cb) -> np.ndarray:
    """(ia|jb) as Om[i,a,j,b] by the reference's four quarter transforms."""
    n = XX.shape[0]
    no1, nv1, no2, nv2 = Ci.shape[1], Ca.shape[1], Cj.shape[1], Cb.shape[1]
    Om = np.zeros(no1 * nv1 * no2 * nv2)
    rc = lib().orc_ao2mo(n, _f(XX), _f(Ci), no1, _f(Ca), nv1, _f(Cj), no2, _f(Cb), nv2, Om)
    if rc != 0:
        raise MemoryError("ao2mo")
    return Om.reshape(no1, nv1, no2, nv2, order="F")


def cis_records(XX: np.ndarray, CA: np.ndarray, CB: np.ndarray, noA: int, noB: int) -> dict:
    """The UHF CIS integral files of slow_ao2mo_CIS_UHF (src/ao2mo/ao2mo.f90:919-1227)
    as lists of records: ajib_AA/AB/BB hold Om(a,i,j,b) = (ai|jb) over the blocks
    (vrt, occ, occ, vrt) (:955-996, :1040-1075, :1077-1113), ajbi_AA/BB hold
    Om(a,b,j,i) over (vrt, vrt, occ, occ) (:1001-1036, :1115-1153); one record per
    (j, b), j outer, with the (i, a) block, a fastest."""
    out = {}
    for name, C1, C3, o1, o3, ajbi in (("ajib_AA", CA, CA, noA, noA, False), ("ajbi_AA", CA, CA, noA, noA, True),
                                       ("ajib_AB", CA, CB, noA, noB, False), ("ajib_BB", CB, CB, noB, noB, False),
                                       ("ajbi_BB", CB, CB, noB, noB, True)):
        occ1, vrt1, occ3, vrt3 = C1[:, :o1], C1[:, o1:], C3[:, :o3], C3[:, o3:]
        if not ajbi:
            Om = ao2mo(XX, vrt1, occ1, occ3, vrt3)       # Om[a, i, j, b]
            recs = [Om[:, :, j, b].flatten(order="F") for j in range(o3) for b in range(vrt3.shape[1])]
        else:
            Om = ao2mo(XX, vrt1, vrt1, occ3, occ3)       # Om[a, b, j, i]
            recs = [Om[:, b, j, :].flatten(order="F") for j in range(o3) for b in range(vrt1.shape[1])]
        out[name] = recs
    return out


def mp2_rhf(eig: np.ndarray, Om: np.ndarray):
    no, nv = Om.shape[0], Om.shape[1]
    out = np.zeros(3)
    lib().orc_mp2_rhf(no, nv, np.ascontiguousarray(eig, dtype=np.float64), _f(Om), out)
    return {"E_AA": out[0], "E_AB": out[1], "E_MP2": out[2]}


def mp2_uhf(eA, eB, OAA, OBB, OAB):
    noA, nvA, noB, nvB = OAA.shape[0], OAA.shape[1], OBB.shape[0], OBB.shape[1]
    out = np.zeros(4)
    lib().orc_mp2_uhf(noA, noB, nvA, nvB, np.ascontiguousarray(eA, dtype=np.float64),
                      np.ascontiguousarray(eB, dtype=np.float64), _f(OAA), _f(OBB), _f(OAB), out)
    return {"E_AA": out[0], "E_BB": out[1], "E_AB": out[2], "E_MP2": out[3]}


def mp2(mol: Molecule, res: SCFResult, XX: np.ndarray):
    """ao2mo + mp2 as the reference's myQC program runs them after scf (myQC.f90:73,84)."""
    if mol.options[3] == 0:
        no = mol.nelcA
        C = res.C
        Om = ao2mo(XX, C[:, :no], C[:, no:], C[:, :no], C[:, no:])
        return mp2_rhf(res.eig, Om)
    noA, noB = mol.nelcA, mol.nelcB
    CA, CB = res.C[0], res.C[1]
    OAA = ao2mo(XX, CA[:, :noA], CA[:, noA:], CA[:, :noA], CA[:, noA:])
    OBB = ao2mo(XX, CB[:, :noB], CB[:, noB:], CB[:, :noB], CB[:, noB:])
    OAB = ao2mo(XX, CA[:, :noA], CA[:, noA:], CB[:, :noB], CB[:, noB:])
    return mp2_uhf(res.eig[0], res.eig[1], OAA, OBB, OAB)


def run_job(zmat_text: str, basis_text: str, ftab: np.ndarray, mode: int = 0, conv_exp: int | None = None):
    """parse -> int1e -> int2e -> scf [-> ao2mo -> mp2], the myQC.f90 stage order."""
    mol = parse_zmat_text(zmat_text)
    basis = parse_mybasis_text(basis_text, mol.atoms)
    S, H = int1e(mol, basis, ftab, mode)
    XX = int2e(mol, basis, ftab, mode)
    res = scf(mol, S, H, XX, conv_exp=conv_exp)
    out = {"mol": mol, "basis": basis, "S": S, "H": H, "XX": XX, "scf": res}
    if mol.options[1] == 1:
        out["mp2"] = mp2(mol, res, XX)
    return out
