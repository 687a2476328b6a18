"""The quartet store (each screened shell quartet once) against the full n^4
array with the same Schwarz threshold: the RHF Fock matrix digested from the
store, the n^4 array filled from it, SCF and MP2 energies, determinism.

Tolerances: G to 1e-12 relative (the two paths sum the same integrals in
different orders, and the bra/ket roles of a quartet may differ, ~1e-16
relative per integral); the filled array to 1e-14 absolute; SCF energies to
1e-10 Eh, MP2 energies to 1e-11 Eh."""
import numpy as np
import pytest

from myqc_gb300 import MODE_REFERENCE, MODE_TIGHT, PREC_FP64, STORE_FULL, STORE_QUARTETS, formats, molecules

pytestmark = pytest.mark.gpu

CO2 = "CARTESIAN\nC 0.00 0.00 0.00\nO 0.00 0.00 -1.16\nO 0.00 0.00 1.16\nEND\n\nCALC= MP2\nBASIS= STO-3G\n" \
      "CHARGE= 0\nMULTI= 1\nREF= RHF\n"


@pytest.fixture
def qctx(ctx):
    yield ctx
    ctx.set_eri_storage(STORE_FULL)
    ctx.set_schwarz(0.0)


def _system(name, basis_text):
    if name == "CO2":
        sysm = formats.parse_zmat_text(CO2)
    else:
        nmol = int(name[len("water"):])
        sysm = molecules.water_cluster_system(nmol, max(3.0, (27.0 * nmol) ** (1 / 3)), 3)
    return sysm, formats.parse_mybasis_text(basis_text, sysm.atoms)


def _density(n, seed=1):
    rng = np.random.default_rng(seed)
    D = rng.standard_normal((n, n)) * 0.1
    return D + D.T


@pytest.mark.parametrize("mode", [MODE_REFERENCE, MODE_TIGHT])
@pytest.mark.parametrize("name", ["CO2", "water2", "water5", "water8"])
def test_store_fock_matches_full(qctx, ftab, basis_text, name, mode):
    sysm, basis = _system(name, basis_text)
    qctx.set_system(sysm, basis, ftab if mode == MODE_REFERENCE else None, mode)
    qctx.set_schwarz(1e-12)
    D = _density(qctx.n)
    qctx.set_eri_storage(STORE_FULL)
    qctx.eri_store()
    Gf = qctx.fock(D)
    qctx.set_eri_storage(STORE_QUARTETS)
    qctx.eri_store()
    assert qctx.stat("store_quartets") > 0 and qctx.stat("store_unique") > 0
    Gq = qctx.fock(D)
    scale = max(1.0, np.max(np.abs(Gf)))
    assert np.max(np.abs(Gq - Gf)) < 1e-12 * scale
    assert np.array_equal(Gq, qctx.fock(D))  # deterministic: bit-identical on a second build
    # the symmetric part is exact by construction
    assert np.max(np.abs(Gq - Gq.T)) == 0.0


@pytest.mark.parametrize("name", ["CO2", "water4"])
def test_store_fills_the_full_array(qctx, basis_text, name):
    """A consumer of the n^4 array (UHF digestion here) gets it filled from the
    store: the same integrals as the full pass with the same threshold."""
    sysm, basis = _system(name, basis_text)
    qctx.set_system(sysm, basis, None, MODE_TIGHT)
    qctx.set_schwarz(1e-12)
    n = qctx.n
    Da, Db = _density(n, 2), _density(n, 3)
    qctx.set_eri_storage(STORE_FULL)
    qctx.eri_store()
    Gaf, Gbf = qctx.fock(Da, Db)
    qctx.set_eri_storage(STORE_QUARTETS)
    qctx.eri_store()
    Gaq, Gbq = qctx.fock(Da, Db)  # UHF: through the filled array
    scale = max(1.0, np.max(np.abs(Gaf)))
    assert np.max(np.abs(Gaq - Gaf)) < 1e-13 * scale and np.max(np.abs(Gbq - Gbf)) < 1e-13 * scale


def test_store_scf_and_mp2(qctx, basis_text):
    sysm, basis = _system("water8", basis_text)
    out = {}
    for st in (STORE_FULL, STORE_QUARTETS):
        qctx.set_system(sysm, basis, None, MODE_TIGHT)
        qctx.set_schwarz(1e-12)
        qctx.set_eri_storage(st)
        S, H = qctx.int1e()
        qctx.eri_store()
        r = qctx.scf(S, H, sysm.nelcA, sysm.nelcB, conv=1e-10, conv_rms=True, diis=8, max_iter=100)
        m = qctx.mp2_rhf(r.eig, sysm.nelcA, PREC_FP64, C=r.C)
        out[st] = (r.energy, m["E_MP2"], r.iterations)
    assert abs(out[STORE_FULL][0] - out[STORE_QUARTETS][0]) < 1e-10
    assert abs(out[STORE_FULL][1] - out[STORE_QUARTETS][1]) < 1e-11
    assert out[STORE_FULL][2] == out[STORE_QUARTETS][2]


def test_store_needs_a_threshold(qctx, basis_text):
    from myqc_gb300 import MyQCError
    sysm, basis = _system("CO2", basis_text)
    qctx.set_system(sysm, basis, None, MODE_TIGHT)
    qctx.set_schwarz(0.0)
    qctx.set_eri_storage(STORE_QUARTETS)
    with pytest.raises(MyQCError):
        qctx.eri_store()


@pytest.mark.parametrize("thr", [0.0, 1e-12])
def test_direct_build_through_the_store(qctx, basis_text, thr):
    """The direct RHF build (no integrals kept between builds) recomputes the
    store's blocks and digests them: no atomics, so two builds agree bit for
    bit, and they agree with the stored full-array build."""
    sysm, basis = _system("water5", basis_text)
    qctx.set_system(sysm, basis, None, MODE_TIGHT)
    qctx.set_schwarz(thr)
    D = _density(qctx.n, 4)
    G1 = qctx.fock(D, direct=True)
    G2 = qctx.fock(D, direct=True)
    assert np.array_equal(G1, G2)
    qctx.set_eri_storage(STORE_FULL)
    qctx.eri_store()
    Gf = qctx.fock(D)
    assert np.max(np.abs(G1 - Gf)) < 1e-12 * max(1.0, np.max(np.abs(Gf)))


@pytest.mark.parametrize("direct", [False, True])
def test_partitions_sum_to_the_full_fock(qctx, basis_text, direct):
    """A molecule split over processes: each part of the quartet store (or of
    the direct build) gives its share of G, and the shares sum to the whole
    G -- here the three parts run one after the other on one GPU."""
    from myqc_gb300 import MyQCError
    sysm, basis = _system("water5", basis_text)
    qctx.set_system(sysm, basis, None, MODE_TIGHT)
    qctx.set_schwarz(1e-12)
    qctx.set_eri_storage(STORE_QUARTETS)
    D = _density(qctx.n, 6)
    if not direct:
        qctx.eri_store()
    G = qctx.fock(D, direct=direct)
    parts = []
    try:
        for k in range(3):
            qctx.set_partition(k, 3)
            if not direct:
                qctx.eri_store()
            parts.append(qctx.fock(D, direct=direct))
        with pytest.raises(MyQCError):  # the SCF of a split molecule iterates on the host
            S, H = qctx.int1e()
            qctx.scf(S, H, sysm.nelcA, sysm.nelcB, conv=1e-8, diis=8, max_iter=5)
    finally:
        qctx.set_partition(0, 1)
    assert all(np.max(np.abs(p)) > 0 for p in parts)
    assert np.max(np.abs(sum(parts) - G)) < 1e-12 * max(1.0, np.max(np.abs(G)))


@pytest.mark.parametrize("name", ["water5", "water16"])
def test_transform_from_the_store(qctx, basis_text, name):
    """The split transform with no n^4 array: its first quarter read straight
    from the quartet store (sparse, FP32 on the CUDA cores), the rest split
    BF16 x3 on the tensor cores, against the FP64 transform of the n^4 array
    filled from the same store: (ia|jb) within 1e-4 of the largest element and
    E(MBPT2) within 1 uEh (the split transform's own bounds); and against the
    split transform of the filled array within 1e-5 relative."""
    from myqc_gb300 import PREC_SPLIT_BF16X3
    sysm, basis = _system(name, basis_text)
    qctx.set_system(sysm, basis, None, MODE_TIGHT)
    qctx.set_schwarz(1e-12)
    qctx.set_eri_storage(STORE_QUARTETS)
    S, H = qctx.int1e()
    qctx.eri_store()
    r = qctx.scf(S, H, sysm.nelcA, sysm.nelcB, conv=1e-10, conv_rms=True, diis=8, max_iter=100)
    no = sysm.nelcA
    C = r.C
    blocks = (C[:, :no], C[:, no:], C[:, :no], C[:, no:])
    got = qctx.ao2mo_iajb(*blocks, PREC_SPLIT_BF16X3)
    m_store = qctx.mp2_rhf(r.eig, no, PREC_SPLIT_BF16X3, C=C)
    n = qctx.n
    qctx.fock(_density(n, 7), _density(n, 8))  # a UHF build fills the n^4 array from the store
    ref = qctx.ao2mo_iajb(*blocks, PREC_FP64)
    split_full = qctx.ao2mo_iajb(*blocks, PREC_SPLIT_BF16X3)
    m64 = qctx.mp2_rhf(r.eig, no, PREC_FP64, C=C)
    big = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) < 1e-4 * big
    assert np.max(np.abs(got - split_full)) < 1e-5 * big
    assert abs(m_store["E_MP2"] - m64["E_MP2"]) < 1e-6, (m_store, m64)


def test_autotuned_integral_launches(qctx, ftab, basis_text):
    """The integral autotuner on (H2O)16 (launches large enough to be tuned):
    every candidate launch shape writes the same integrals, so the store --
    and the Fock matrix digested from it -- is bit-identical whether the pass
    ran with the defaults, while tuning, or with the tuned choices; the
    report lists each tuned signature with its chosen candidate.  The survivor
    counts (primitive quartets) match between the passes."""
    sysm, basis = _system("water16", basis_text)
    qctx.set_system(sysm, basis, ftab, MODE_REFERENCE)
    qctx.set_schwarz(1e-12)
    qctx.set_eri_storage(STORE_QUARTETS)
    D = _density(qctx.n, 7)
    qctx.set_eri_tuning(0)
    qctx.eri_store()
    G0 = qctx.fock(D)
    prims0 = qctx.stat("prim_quartets")
    qctx.set_eri_tuning(1)
    qctx.eri_store()  # tunes: each candidate runs once
    G1 = qctx.fock(D)
    rep = qctx.eri_tuning_report()
    qctx.eri_store()  # the tuned choices
    G2 = qctx.fock(D)
    assert np.array_equal(G0, G1) and np.array_equal(G0, G2)
    assert qctx.stat("prim_quartets") == prims0
    lines = [ln for ln in rep.splitlines() if ln.strip()]
    assert lines and all("*" in ln for ln in lines), rep
    assert any("binned" in ln and "plain" in ln for ln in lines), rep


@pytest.mark.parametrize("name", ["water8", "water16"])
def test_screened_increments(qctx, basis_text, name):
    """Screened FP64 increments (after the first build, G_k = G_(k-1) +
    G[D_k - D_(k-1)] over the quartets with Q_P Q_Q max|dD| >= 1e-12) against
    full builds from the same store: the SCF energy to 1e-10 Eh, the MP2 energy
    to 1e-10 Eh, the same iteration count within one; every build after the
    first is an increment."""
    sysm, basis = _system(name, basis_text)
    qctx.set_system(sysm, basis, None, MODE_TIGHT)
    qctx.set_schwarz(1e-12)
    qctx.set_eri_storage(STORE_QUARTETS)
    S, H = qctx.int1e()
    qctx.eri_store()
    out = {}
    try:
        for tau in (0.0, 1e-12):
            qctx.set_fock_screened_increments(tau)
            r = qctx.scf(S, H, sysm.nelcA, sysm.nelcB, conv=1e-10, conv_rms=True, diis=8, max_iter=100)
            m = qctx.mp2_rhf(r.eig, sysm.nelcA, PREC_FP64, C=r.C)
            out[tau] = (r.energy, m["E_MP2"], r.iterations, qctx.stat("fock_screened_builds"),
                        qctx.stat("fock_full_builds"))
    finally:
        qctx.set_fock_screened_increments(0.0)
    full, inc = out[0.0], out[1e-12]
    assert abs(full[0] - inc[0]) < 1e-10, (full, inc)
    assert abs(full[1] - inc[1]) < 1e-10, (full, inc)
    assert abs(full[2] - inc[2]) <= 1
    assert full[3] == 0 and inc[4] == 1 and inc[3] == inc[2] - 1
