"""Host-side formats and the C ABI boundary (no GPU needed)."""
import ctypes
import glob
import os

import numpy as np
import pytest

import oracle as O
from conftest import ROOT, golden
from myqc_gb300 import _lib, formats, molecules


@pytest.mark.parametrize("path", sorted(glob.glob(golden("zmat", "*.ZMAT"))))
def test_zmat_and_basis_match_oracle(path, basis_text):
    t = open(path).read()
    a, b = formats.parse_zmat_text(t), O.parse_zmat_text(t)
    assert np.array_equal(a.atoms, b.atoms) and np.array_equal(a.xyz, b.xyz)
    assert a.options == b.options and (a.nelcA, a.nelcB) == (b.nelcA, b.nelcB)
    ba, bb = formats.parse_mybasis_text(basis_text, a.atoms), O.parse_mybasis_text(basis_text, b.atoms)
    for k in ("bas", "set", "basinfo", "setinfo"):
        assert np.array_equal(getattr(ba, k), getattr(bb, k))


def test_env_files_round_trip(tmp_path):
    s = formats.parse_zmat_text(open(golden("zmat", "NO.ZMAT")).read())
    formats.write_env(s, str(tmp_path))
    r = formats.read_env(str(tmp_path))
    assert np.array_equal(r.atoms, s.atoms) and np.array_equal(r.xyz, s.xyz)
    assert r.options == s.options and (r.nelcA, r.nelcB) == (s.nelcA, s.nelcB)


def test_ftab_reader(ftab):
    assert np.array_equal(formats.read_ftab(golden("Ftab")), ftab)


def test_records_and_subrecords(tmp_path, monkeypatch):
    a = np.arange(1000, dtype=np.float64).reshape(10, 100)
    b = np.ones((3, 3))
    p = str(tmp_path / "rec")
    formats.write_records(p, [a, b])
    r = formats.read_records(p)
    assert np.array_equal(np.frombuffer(r[0]).reshape(10, 100, order="F"), a)
    assert np.array_equal(np.frombuffer(r[1]).reshape(3, 3), b)
    # a record longer than one subrecord: split with negated continuation markers
    monkeypatch.setattr(formats, "MAX_SUBRECORD", 2400)
    formats.write_records(p, [a])
    raw = open(p, "rb").read()
    assert len(raw) == 8000 + 8 * 4  # ceil(8000/2400) = 4 subrecords
    assert np.frombuffer(raw[:4], "<i4")[0] == -2400
    assert np.array_equal(np.frombuffer(formats.read_records(p)[0]).reshape(10, 100, order="F"), a)


def test_water_cluster_generator():
    s1 = molecules.water_cluster_system(32, 9.5, 0)
    s2 = molecules.water_cluster_system(32, 9.5, 0)
    assert np.array_equal(s1.xyz, s2.xyz)
    assert s1.nelcA == s1.nelcB == 160
    o = s1.xyz[s1.atoms == 8] / formats.A2B
    d = np.linalg.norm(o[:, None] - o[None], axis=-1)
    assert np.min(d[d > 0]) >= 2.7 - 1e-12
    for k in range(32):
        w = s1.xyz[3 * k: 3 * k + 3] / formats.A2B
        assert abs(np.linalg.norm(w[1] - w[0]) - 0.9572) < 1e-12
        cosang = np.dot(w[1] - w[0], w[2] - w[0]) / 0.9572 ** 2
        assert abs(np.degrees(np.arccos(cosang)) - 104.52) < 1e-9


def test_header_symbols_exported():
    """libmyqc.so loads and exports every function include/myqc.h declares."""
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libmyqc.so not built")
    L = ctypes.CDLL(_lib.LIB_PATH)
    names = _lib.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert ctypes.CDLL(_lib.LIB_PATH).mq_version  # callable without a GPU
    L.mq_version.restype = ctypes.c_char_p
    assert b"sm_103a" in L.mq_version()


def test_fortran_module_binds_every_entry_point():
    """The Fortran interface module include/myqc_gpu.f90 has one BIND(C)
    interface per function include/myqc.h declares, and no other."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    text = open(os.path.join(root, "include", "myqc_gpu.f90")).read()
    module = text[text.index("MODULE myqc_gpu"):text.index("END MODULE")]
    bound = set(re.findall(r"FUNCTION (mq_\w+)\(", module))
    assert bound == set(_lib.header_symbols()), (set(_lib.header_symbols()) ^ bound)
