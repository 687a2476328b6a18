"""The reference's file formats (jhthorpe/myQC), so that the drop-ins read and
write exactly what its programs do.

* ZMAT (CARTESIAN input) -> atoms, bohr coordinates, options, electron counts:
  src/parser/parser.f90:435-547 (build), :622-678 (cartesian), :683-735
  (read_options); envdat / nucpos / fmem as it writes them (:490-530).
* mybasis -> the flat bas / set / basinfo / setinfo arrays of buildBasis
  (src/myQC/basis.f90:23-226).
* Ftab: one gfortran sequential unformatted record of Ft(0:120,0:22)
  (src/integrals/int2e.f90:160-163).
* gfortran sequential unformatted records (XX, Da, Dold, Guv, ijab_*): each
  record is <int32 length> payload <int32 length>.  A record longer than
  2**31-9 bytes is written as subrecords whose leading marker is negated when
  another subrecord follows and whose trailing marker is negated when a
  subrecord precedes it (libgfortran's layout).
* List-directed text matrices (Huv, Suv, Cui, eig): whitespace-separated
  numbers, column-major.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

A2B = 1.8897161646320724  # parser.f90:14
ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne"]
MASS = [1.0, 4.0, 7.0, 9.0, 11.0, 12.0, 14.0, 16.0, 19.0, 20.0]  # parser.f90:472 (integer masses)
DEFAULT_OPTIONS = [0, 0, 0, 0, 0, 1, 1000, 1, 7, 0, 1, 0, 1, 0, 0, 0, 0]
MAX_SUBRECORD = 2147483639  # 2**31 - 9 bytes


@dataclass
class System:
    atoms: np.ndarray            # int32 Z
    xyz: np.ndarray              # (nnuc, 3) bohr
    nelcA: int
    nelcB: int
    options: list = field(default_factory=lambda: list(DEFAULT_OPTIONS))

    @property
    def uhf(self) -> bool:
        return self.options[3] == 1


@dataclass
class BasisArrays:
    bas: np.ndarray
    set: np.ndarray
    basinfo: np.ndarray
    setinfo: np.ndarray

    @property
    def norb(self) -> int:
        return int(self.basinfo[1])


# ------------------------------------------------------------------ ZMAT
def _i8(tok: str) -> int:
    s = tok[:8].strip()  # READ(chr,'(I8)')
    return int(s) if s else 0


def parse_zmat_text(text: str) -> System:
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    if not lines or not lines[0].split() or lines[0].split()[0] != "CARTESIAN":
        raise ValueError("ZMAT: only CARTESIAN geometry input is supported")
    atoms, xyz = [], []
    i = 1
    while True:
        if i >= len(lines):
            raise ValueError("ZMAT: missing END marker")
        tok = lines[i].split()
        if tok and tok[0] == "END":
            break
        if not tok or tok[0] not in ELEMENTS:
            raise ValueError(f"ZMAT: bad atom line {lines[i]!r}")
        atoms.append(ELEMENTS.index(tok[0]) + 1)
        xyz.append([float(t.replace("D", "E").replace("d", "e")) for t in tok[1:4]])
        i += 1
    opts = list(DEFAULT_OPTIONS)
    nline = len(atoms) + 2
    for ln in lines[nline + 1: len(lines)]:
        tok = ln.split()
        if len(tok) < 2:
            continue
        k, v = tok[0], tok[1]
        if k == "CALC=":
            opts[1] = {"SCF": 0, "HF": 0, "MP2": 1, "CIS": 2}[v]
        elif k == "BASIS=":
            opts[2] = {"STO-3G": 0, "tester1": 1, "tester2": 2, "tester3": 3}[v]
        elif k == "REF=":
            if v not in ("RHF", "UHF"):
                raise ValueError("ZMAT: only RHF and UHF references")
            opts[3] = 0 if v == "RHF" else 1
        elif k == "PAR=":
            opts[4] = {"OMP": 2, "MPI": 3}.get(v, 1)
        elif k == "NODES=":
            opts[5] = 1
        elif k == "MEMORY=":
            opts[6] = max(_i8(v), 0) if _i8(v) >= 0 else 1000
        elif k == "VERB=":
            opts[7] = {"1": 1, "2": 2, "3": 3}.get(v, 0)
        elif k == "SCF_Conv=":
            opts[8] = _i8(v)
        elif k == "CHARGE=":
            opts[9] = _i8(v)
        elif k == "MULTI=":
            m = _i8(v)
            if m <= 0:
                raise ValueError("ZMAT: bad multiplicity")
            opts[10] = m
        elif k == "UNITS=":
            opts[11] = 1 if v == "Bohr" else 0
        elif k == "AO2MO=":
            opts[12] = 1
        elif k == "EXCITE=":
            opts[13] = 1 if v in ("CIS", "1") else 0
        elif k == "ROOT_ALG=":
            opts[14] = 0
        elif k == "E_NUM=":
            opts[15] = 1 if _i8(v) < 0 else _i8(v)
        elif k == "PROP=":
            opts[16] = {"FIRST": 1, "1": 1, "SECOND": 2, "2": 2}.get(v, 0)
    Z = np.array(atoms, dtype=np.int32)
    X = np.array(xyz, dtype=np.float64).reshape(-1, 3)
    m = np.array([MASS[z - 1] for z in Z])
    com = np.zeros(3)
    tot = 0.0
    for a in range(len(Z)):
        com = com + m[a] * X[a]
        tot = tot + m[a]
    X = X - com / tot
    if opts[11] == 0:
        X = X * A2B
    nelc = int(Z.sum()) - opts[9]
    unpr = opts[10] - 1
    half = int((nelc - unpr) / 2)
    return System(atoms=Z, xyz=X, nelcA=half + unpr, nelcB=half, options=opts)


def system_from_geometry(symbols, xyz_angstrom, charge=0, multiplicity=1, uhf=False, calc_mp2=True) -> System:
    """Build a System the way parse would for a CARTESIAN ZMAT in Angstrom."""
    lines = ["CARTESIAN"] + [f"{s} {float(x)!r} {float(y)!r} {float(z)!r}"
                             for s, (x, y, z) in zip(symbols, xyz_angstrom)]
    lines += ["END", "", f"CALC= {'MP2' if calc_mp2 else 'SCF'}", "BASIS= STO-3G", f"CHARGE= {charge}",
              f"MULTI= {multiplicity}", f"REF= {'UHF' if uhf else 'RHF'}"]
    return parse_zmat_text("\n".join(lines) + "\n")


def write_env(sysm: System, folder: str = ".") -> None:
    """envdat, nucpos, fmem as parse writes them (parser.f90:490-530)."""
    import os
    with open(os.path.join(folder, "nucpos"), "w") as f:
        for z, (x, y, w) in zip(sysm.atoms, sysm.xyz):
            f.write(f" {int(z):11d} {float(x)!r:>25} {float(y)!r:>25} {float(w)!r:>25}\n")
    with open(os.path.join(folder, "envdat"), "w") as f:
        f.write(f" {len(sysm.atoms):11d}\n {sysm.nelcA:11d} {sysm.nelcB:11d}\n {len(sysm.options):11d}\n")
        f.write(" " + " ".join(f"{o:20d}" for o in sysm.options) + "\n\n")
        f.write(" #number of nuclei\n #number of electrons\n #length of options array\n options array\n")
    with open(os.path.join(folder, "fmem"), "w") as f:
        f.write(f" {sysm.options[6]:20d}\n")


def read_env(folder: str = ".") -> System:
    """getenv (src/myQC/env.f90:16-74)."""
    import os
    tok = open(os.path.join(folder, "envdat")).read().split()
    nnuc, nA, nB, nopt = int(tok[0]), int(tok[1]), int(tok[2]), int(tok[3])
    opts = [int(t) for t in tok[4: 4 + nopt]]
    rows = [ln.split() for ln in open(os.path.join(folder, "nucpos")) if ln.strip()][:nnuc]
    Z = np.array([int(r[0]) for r in rows], dtype=np.int32)
    X = np.array([[float(v.replace("D", "E")) for v in r[1:4]] for r in rows])
    return System(atoms=Z, xyz=X, nelcA=nA, nelcB=nB, options=opts)


# ------------------------------------------------------------------ mybasis
def parse_mybasis_text(text: str, atoms, key: str = "STO-3G") -> BasisArrays:
    rows = [ln.split() for ln in text.split("\n")]
    first = [r[0][:8] if r else "" for r in rows]
    p = first.index(key)
    Smax, Cmax, Omax, almax, OpS = (int(x) for x in rows[p + 1][:5])
    n_atoms = len(atoms)
    setl = 3 + OpS
    bas = np.zeros(n_atoms * almax * OpS)
    sets = np.zeros(n_atoms * almax)
    basinfo = np.zeros(2 + 5 * Omax * n_atoms, dtype=np.int32)
    setinfo = np.zeros(2 + n_atoms * almax * setl, dtype=np.int32)
    setnum = orbnum = 0
    for i, Z in enumerate(atoms):
        name = ELEMENTS[int(Z) - 1]
        q = p
        while first[q] != name:
            q += 1
        sec, orb, nset = (int(x) for x in rows[q + 1][:3])
        q += 2
        basinfo[0] = OpS
        basinfo[1] += orb
        setinfo[0] += nset
        setinfo[1] = setl
        for _ in range(sec):
            func, coef, pri, ang, ori = (int(x) for x in rows[q][:5])
            q += 1
            for _k in range(func):
                v = [float(t.replace("D", "E")) for t in rows[q][: coef + 1]]
                q += 1
                t = v[coef]
                sid = setnum + int(np.floor(abs(t) + 0.5)) * (1 if t >= 0 else -1)
                sets[sid] = v[coef - 1]
                base = 1 + sid * setl
                k = int(setinfo[base + 1])
                setinfo[base + 3] = i
                if ori == -1:
                    setinfo[base + 4 + k] = orbnum
                    bas[k + sid * OpS] = v[0]
                    k += 1
                elif ori == 2:
                    for m in range(3):
                        setinfo[base + 4 + k] = orbnum + m
                        bas[k + sid * OpS] = v[0]
                        k += 1
                    setinfo[base + 2] = max(setinfo[base + 2], 1)
                else:
                    raise ValueError("mybasis: only s and p sections are supported")
                setinfo[base + 1] = k
            if ori == -1:
                basinfo[2 + 5 * orbnum: 7 + 5 * orbnum] = [pri, ang, ori, func, i]
                orbnum += 1
            else:
                for m in range(3):
                    basinfo[2 + 5 * (orbnum + m): 7 + 5 * (orbnum + m)] = [pri, ang, m, func, i]
                orbnum += 3
        setnum = int(setinfo[0])
    return BasisArrays(bas=bas, set=sets, basinfo=basinfo, setinfo=setinfo)


# ------------------------------------------------------------------ Fortran records
def write_records(path: str, arrays) -> None:
    with open(path, "wb") as f:
        for a in arrays:
            data = np.asfortranarray(a).tobytes(order="F")
            n = len(data)
            if n <= MAX_SUBRECORD:
                f.write(struct.pack("<i", n) + data + struct.pack("<i", n))
                continue
            pos = 0
            first = True
            while pos < n:
                m = min(MAX_SUBRECORD, n - pos)
                more = pos + m < n
                f.write(struct.pack("<i", -m if more else m))
                f.write(data[pos: pos + m])
                f.write(struct.pack("<i", m if first else -m))
                pos += m
                first = False


def read_records(path: str) -> list[bytes]:
    out = []
    with open(path, "rb") as f:
        raw = f.read()
    pos = 0
    while pos < len(raw):
        chunks = []
        while True:
            (m,) = struct.unpack("<i", raw[pos: pos + 4])
            L = abs(m)
            chunks.append(raw[pos + 4: pos + 4 + L])
            pos += 8 + L
            if m >= 0:
                break
        out.append(b"".join(chunks))
    return out


def read_ftab(path: str) -> np.ndarray:
    recs = read_records(path)
    if len(recs) != 1 or len(recs[0]) != 121 * 23 * 8:
        raise ValueError("Ftab: expected one record of 121x23 doubles")
    return np.frombuffer(recs[0], "<f8").copy()


def read_text_numbers(path: str) -> np.ndarray:
    return np.array([float(t.replace("D", "E")) for t in open(path).read().split()])


def write_text_matrix(path: str, mats) -> None:
    """List-directed style: 17 significant digits, column-major, one line per matrix."""
    with open(path, "w") as f:
        for m in mats:
            f.write(" " + " ".join(f"{v: .16E}" for v in np.asarray(m).reshape(-1, order="F")) + "\n")
