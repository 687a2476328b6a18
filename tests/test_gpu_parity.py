"""GPU path vs the CPU oracle on the reference's own examples.

Tolerances: ERIs 1e-10 Eh absolute, SCF total energy 1e-9 Eh,
MP2 correlation energy 1e-8 Eh; one-electron integrals and Fock matrices
1e-11.  Mode 0 compares against the restatement of the reference (oracle A),
mode 1 against the tight FP64 oracle (oracle B)."""
import numpy as np
import pytest

import oracle as O
from conftest import golden
from myqc_gb300 import formats
from myqc_gb300.session import run_job

pytestmark = pytest.mark.gpu

EXAMPLES = ["Be", "O_singlet", "NO", "CO2", "HeH", "OH", "H2", "HF", "CO", "O_triplet", "H"]
CO2_CONFIG = "CARTESIAN\nC 0.00 0.00 0.00\nO 0.00 0.00 -1.16\nO 0.00 0.00 1.16\nEND\n\nCALC= MP2\nBASIS= STO-3G\n" \
             "CHARGE= 0\nMULTI= 1\nREF= RHF\n"


def _zmat(name):
    return open(golden("zmat", name + ".ZMAT")).read()


def _setup(ctx, ztext, btext, ftab, mode):
    sysm = formats.parse_zmat_text(ztext)
    basis = formats.parse_mybasis_text(btext, sysm.atoms)
    ctx.set_system(sysm, basis, ftab, mode)
    mol = O.parse_zmat_text(ztext)
    ob = O.parse_mybasis_text(btext, mol.atoms)
    return sysm, basis, mol, ob


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", EXAMPLES + ["CO2_116"])
def test_integrals(ctx, ftab, basis_text, name, mode):
    zt = CO2_CONFIG if name == "CO2_116" else _zmat(name)
    sysm, basis, mol, ob = _setup(ctx, zt, basis_text, ftab, mode)
    S, H = ctx.int1e()
    So, Ho = O.int1e(mol, ob, ftab, mode)
    assert np.max(np.abs(S - So)) < 1e-11
    assert np.max(np.abs(H - Ho)) < 1e-10
    # dipole integrals (int1p)
    P = ctx.int1p()
    assert np.max(np.abs(P - O.int1p(mol, ob, mode))) < 1e-11
    XX = ctx.eri_full()
    XXo = O.int2e(mol, ob, ftab, mode)
    assert np.max(np.abs(XX - XXo)) < 1e-10
    # stored Fock build on a random symmetric density
    rng = np.random.default_rng(1)
    n = S.shape[0]
    D = rng.standard_normal((n, n))
    D = D + D.T
    G = ctx.fock(D)
    assert np.max(np.abs(G - O.fock_rhf(XXo, D))) < 1e-11 * max(1.0, np.max(np.abs(G)))
    Db = rng.standard_normal((n, n))
    Db = Db + Db.T
    Ga, Gb = ctx.fock(D, Db)
    Gao, Gbo = O.fock_uhf(XXo, D, Db)
    assert np.max(np.abs(Ga - Gao)) < 1e-11 * max(1.0, np.max(np.abs(Ga)))
    assert np.max(np.abs(Gb - Gbo)) < 1e-11 * max(1.0, np.max(np.abs(Gb)))
    # direct build (integrals recomputed and digested in one kernel)
    Gd = ctx.fock(D, direct=True)
    assert np.max(np.abs(Gd - G)) < 1e-11 * max(1.0, np.max(np.abs(G)))


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", EXAMPLES + ["CO2_116"])
def test_scf_mp2(ctx, ftab, basis_text, name, mode):
    zt = CO2_CONFIG if name == "CO2_116" else _zmat(name)
    sysm = formats.parse_zmat_text(zt)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ref = O.run_job(zt, basis_text, ftab, mode, conv_exp=11)
    out = run_job(sysm, basis, ftab, mode, conv=1e-11, ctx=ctx, mp2=True)
    assert abs(out["scf"].energy - ref["scf"].energy) < 1e-9
    assert np.max(np.abs(out["scf"].eig - ref["scf"].eig)) < 1e-8
    refmp2 = ref.get("mp2") or O.mp2(ref["mol"], ref["scf"], ref["XX"])
    assert abs(out["mp2"]["E_MP2"] - refmp2["E_MP2"]) < 1e-8


def test_molden_pins(ctx, ftab, basis_text):
    """The reference's own MOLDEN orbital energies, reproduced on the GPU."""
    import json
    pins = json.load(open(golden("reference_pins.json")))["molden"]
    for name, tol in (("Be", 2e-8), ("O_singlet", 2e-8), ("NO", 1.5e-7)):
        sysm = formats.parse_zmat_text(_zmat(name))
        basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
        out = run_job(sysm, basis, ftab, 0, ctx=ctx, mp2=False)
        eig = out["scf"].eig
        if sysm.uhf:
            assert np.max(np.abs(eig[0] - pins[name]["alpha"])) < tol
            assert np.max(np.abs(eig[1] - pins[name]["beta"])) < tol
        else:
            assert np.max(np.abs(eig - pins[name]["alpha"])) < tol


def test_syev_batched(ctx):
    rng = np.random.default_rng(3)
    for n, batch in ((5, 3), (37, 4), (120, 2), (150, 1)):
        A = rng.standard_normal((batch, n, n))
        A = A + A.transpose(0, 2, 1)
        w, V = ctx.syev_batched(A)
        for b in range(batch):
            assert np.allclose(w[b], np.linalg.eigvalsh(A[b]), atol=1e-12 * n)
            assert np.allclose(A[b] @ V[b], V[b] * w[b], atol=1e-11 * n)


def test_eri_mixed_precision(ctx, basis_text):
    """Quartets with a Schwarz bound below tau computed in FP32: every integral
    of (H2O)8 within 1e-6 tau of the FP64 pass (tau = 1e-3, 1e-4 and 1e-6), the
    FP32 share counted, and FP64 again once tau is 0."""
    from myqc_gb300 import MODE_TIGHT, molecules
    sysm = molecules.water_cluster_system(8, 7.0, 3)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    try:
        ctx.set_schwarz(1e-12)
        ctx.set_eri_mixed(0.0)
        X64 = ctx.eri_full()
        assert ctx.stat("quartets_f32") == 0
        for tau in (1e-3, 1e-4, 1e-6):
            ctx.set_eri_mixed(tau)
            Xm = ctx.eri_full()
            nf = ctx.stat("quartets_f32")
            assert 0 < nf < ctx.stat("quartets")
            err = np.max(np.abs(Xm - X64))
            assert err < 1e-6 * tau, (tau, err)
        ctx.set_eri_mixed(0.0)
        assert np.array_equal(ctx.eri_full(), X64)
    finally:
        ctx.set_eri_mixed(0.0)
        ctx.set_schwarz(0.0)


def test_fock_skips_screened_slabs(ctx, basis_text):
    """With a Schwarz threshold the integral pass marks slabs XX(:,:,i,j) whose
    quartets were all screened out; the digestion skips them.  G must equal,
    bit for bit, G from the same integrals uploaded (every slab read)."""
    from myqc_gb300 import MODE_TIGHT, molecules
    sysm = molecules.water_cluster_system(8, 9.0, 5)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    try:
        ctx.set_schwarz(1e-9)
        XX = ctx.eri_full()
        frac = ctx.stat("live_slabs")
        assert 0.0 < frac < 1.0, frac
        n = ctx.n
        rng = np.random.default_rng(8)
        D = rng.standard_normal((n, n))
        D = D + D.T
        for prec in (0, 1):
            ctx.set_fock_precision(prec)
            G_skip = ctx.fock(D)
            ctx.eri_upload(XX)
            assert ctx.stat("live_slabs") == 1.0
            G_all = ctx.fock(D)
            assert np.array_equal(G_skip, G_all), prec
            ctx.eri_store()
    finally:
        ctx.set_fock_precision(0)
        ctx.set_schwarz(0.0)


def test_dgemm_small_and_large(ctx):
    """mq_dgemm: the library's split-K FP64 kernel (small orders) and cuBLAS
    (large) against NumPy, every transpose case, alpha/beta, odd sizes."""
    rng = np.random.default_rng(6)
    for (m, n, k) in ((1, 1, 1), (5, 7, 3), (33, 17, 65), (224, 224, 224), (150, 64, 300), (1100, 1000, 40)):
        for ta in "NT":
            for tb in "NT":
                A = rng.standard_normal((k, m) if ta == "T" else (m, k))
                B = rng.standard_normal((n, k) if tb == "T" else (k, n))
                C0 = rng.standard_normal((m, n))
                ref = 0.7 * ((A.T if ta == "T" else A) @ (B.T if tb == "T" else B)) - 1.3 * C0
                out = ctx.dgemm(A, B, ta, tb, alpha=0.7, beta=-1.3, C=C0)
                assert np.max(np.abs(out - ref)) < 1e-13 * k * max(1.0, np.max(np.abs(ref)))
    # beta = 0 ignores C (NaN in C must not leak)
    A = rng.standard_normal((40, 30))
    out = ctx.dgemm(A, A, "T", "N", C=np.full((30, 30), np.nan))
    assert np.allclose(out, A.T @ A, atol=1e-12)


def test_syev_cluster_refined(ctx):
    """Orders 111..512 without start vectors take the FP32 cluster Jacobi, the
    FP64 first-order refinement and the FP64 Jacobi.  Spectra: random, and
    bands of near-degenerate levels (gaps down to ~1e-6 of the norm) like a
    molecular cluster's Fock matrix.  Eigenvalues within 1e-13 of the
    norm, orthonormal vectors, residual ||A V - V w|| within 1e-12 of the norm."""
    rng = np.random.default_rng(5)
    cases = []
    for n in (111, 224, 333):
        M = rng.standard_normal((n, n))
        cases.append(M + M.T)
    n = 224
    bands = [(-20.55, 0.02), (-1.35, 0.08), (-0.72, 0.1), (-0.55, 0.1), (-0.45, 0.1)]
    w0 = np.concatenate([c + s * rng.random(32) for c, s in bands] + [0.6 + 0.4 * rng.random(64)])
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (Q * w0) @ Q.T
    cases.append(0.5 * (A + A.T))
    for A in cases:
        n = A.shape[0]
        w, V = ctx.syev_batched(A[None])
        w, V = w[0], V[0]
        nrm = np.linalg.norm(A, 2)
        assert np.max(np.abs(w - np.linalg.eigvalsh(A))) < 1e-13 * nrm * np.sqrt(n)
        assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-13
        assert np.max(np.abs(A @ V - V * w)) < 1e-12 * nrm
        assert np.all(np.diff(w) >= 0)
    assert ctx.stat("eig_cluster") in (8, 16)


def test_fock_water_cluster(ctx, basis_text):
    """Stored Fock build at a size where the digestion's long sums matter:
    (H2O)8, n = 56, tight integrals, a random symmetric density and a
    converged-like one.  G must be symmetric to the last bit and match the
    FP64 contraction of the same XX to 1e-12 relative."""
    from myqc_gb300 import MODE_TIGHT, molecules
    sysm = molecules.water_cluster_system(8, 7.0, 3)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    XX = ctx.eri_full()
    n = ctx.n
    X4 = XX.reshape((n, n, n, n), order="F")
    rng = np.random.default_rng(4)
    for D in (rng.standard_normal((n, n)), rng.random((n, n)) * 0.2):
        D = D + D.T
        G = ctx.fock(D)
        ref = np.einsum("ijkl,kl->ij", X4, D) - 0.5 * np.einsum("ikjl,kl->ij", X4, D)
        assert np.array_equal(G, G.T)
        err = np.max(np.abs(G - ref)) / np.max(np.abs(ref))
        assert err < 1e-12, err


@pytest.mark.parametrize("name", ["CO2", "HF", "NO", "O_triplet", "Be", "(H2O)4"])
def test_scf_purification_same_fixed_point(ctx, ftab, basis_text, name):
    """Density by purification instead of the eigensolver: same energies,
    same iteration count under plain Roothaan (the iterates are the same
    densities), same orbital energies from the final eigensolve.  Open-shell
    cases with degenerate frontier levels take the eigensolver fallback."""
    from myqc_gb300 import molecules
    if name.startswith("("):
        sysm = molecules.water_cluster_system(4, 5.0, 11)
    else:
        sysm = formats.parse_zmat_text(_zmat(name))
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, ftab, 0)
    S, H = ctx.int1e()
    ctx.eri_store()
    for diis in (0, 8):
        a = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, uhf=sysm.uhf, conv=1e-10, diis=diis)
        b = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, uhf=sysm.uhf, conv=1e-10, diis=diis, purify=True)
        assert abs(a.energy - b.energy) < 1e-10, (diis, a.energy, b.energy)
        assert np.max(np.abs(np.asarray(a.eig) - np.asarray(b.eig))) < 1e-8
        assert np.max(np.abs(a.D - b.D)) < 1e-8
        if diis == 0:
            assert abs(a.iterations - b.iterations) <= 1, (a.iterations, b.iterations)


def test_fock_double_float_matches_fp64(ctx, basis_text):
    """The opt-in double-float digestion against the default FP64 one, RHF and
    UHF, on (H2O)6 (n = 42): 1e-12 relative."""
    from myqc_gb300 import FOCK_DF32, FOCK_FP64, MODE_TIGHT, molecules
    sysm = molecules.water_cluster_system(6, 6.5, 5)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    ctx.eri_store()
    n = ctx.n
    rng = np.random.default_rng(8)
    Da, Db = (rng.random((n, n)) * 0.2 for _ in range(2))
    Da, Db = Da + Da.T, Db + Db.T
    ctx.set_fock_precision(FOCK_FP64)
    G64 = ctx.fock(Da)
    Ga64, Gb64 = ctx.fock(Da, Db)
    ctx.set_fock_precision(FOCK_DF32)
    try:
        G32 = ctx.fock(Da)
        Ga32, Gb32 = ctx.fock(Da, Db)
    finally:
        ctx.set_fock_precision(FOCK_FP64)
    for a, b in ((G32, G64), (Ga32, Ga64), (Gb32, Gb64)):
        assert np.max(np.abs(a - b)) < 1e-12 * np.max(np.abs(b))


def test_schwarz_screened_integrals(ctx, basis_text):
    """Schwarz screening at 1e-12 (quartet lists compacted before the integral
    launches): every dropped integral is below the bound, kept ones are
    unchanged, and the direct Fock build from the screened quartets matches
    the stored unscreened one."""
    from myqc_gb300 import MODE_TIGHT, molecules
    sysm = molecules.water_cluster_system(8, 8.0, 2)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_schwarz(0.0)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    XX = ctx.eri_full()
    n = ctx.n
    rng = np.random.default_rng(9)
    D = rng.random((n, n)) * 0.1
    D = D + D.T
    G = ctx.fock(D)
    try:
        ctx.set_schwarz(1e-12)
        XXs = ctx.eri_full()
        nq = ctx.stat("quartets")
        Gd = ctx.fock(D, direct=True)
    finally:
        ctx.set_schwarz(0.0)
    kept = XXs != 0.0
    assert np.array_equal(XXs[kept], XX[kept])
    assert np.max(np.abs(XX[~kept])) < 1e-11
    assert nq > 0
    assert np.max(np.abs(Gd - G)) < 1e-9 * np.max(np.abs(G))


@pytest.mark.parametrize("uhf", [False, True])
def test_incremental_fock_builds(ctx, basis_text, uhf):
    """FP32 incremental Fock builds (mq_set_fock_incremental) once the density
    moves by less than 1e-6, 1e-3 and, the largest threshold allowed, 1e-2: the
    converged energy of full FP64 builds within 1e-8 Eh (the FP32 rounding of
    each increment is never corrected by a later full build, so it adds up over
    the increments: these options are not FP64-accurate and stay out of the
    headline arm), same iteration count within 1, and some builds were
    incremental.  RHF on (H2O)8 (n = 56), UHF on its cation."""
    from myqc_gb300 import FOCK_DF32, FOCK_FP64, MODE_TIGHT, molecules
    sysm = molecules.water_cluster_system(8, 8.0, 11)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_schwarz(0.0)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    S, H = ctx.int1e()
    ctx.eri_store()
    na, nb = (sysm.nelcA, sysm.nelcB) if not uhf else (sysm.nelcA, sysm.nelcB - 1)
    kw = dict(uhf=uhf, conv=1e-10, conv_rms=True, diis=8, max_iter=200)
    ctx.set_fock_precision(FOCK_FP64)
    ref = ctx.scf(S, H, na, nb, **kw)
    try:
        for prec, tau in ((FOCK_FP64, 1e-6), (FOCK_DF32, 1e-6), (FOCK_DF32, 1e-3), (FOCK_DF32, 1e-2)):
            ctx.set_fock_precision(prec)
            ctx.set_fock_incremental(tau)
            r = ctx.scf(S, H, na, nb, **kw)
            assert ctx.stat("fock_inc_builds") >= 2
            assert abs(r.energy - ref.energy) < 1e-8, (prec, r.energy - ref.energy)
            assert abs(r.iterations - ref.iterations) <= 1, (r.iterations, ref.iterations)
    finally:
        ctx.set_fock_incremental(0.0)
        ctx.set_fock_precision(FOCK_FP64)


def test_purification_early_eigensolve(ctx, basis_text):
    """(H2O)16 (n = 112, above the single-CTA Jacobi size): with purification the
    cold eigensolve of a Fock matrix near convergence runs on a second stream
    while the SCF finishes, and the final eigensolve starts from its vectors.
    Energy, orbital energies and density match the eigensolver SCF; MP2 from
    the final orbitals matches too."""
    from myqc_gb300 import MODE_TIGHT, PREC_FP64, molecules
    sysm = molecules.water_cluster_system(16, 7.6, 3)
    basis = formats.parse_mybasis_text(basis_text, sysm.atoms)
    ctx.set_schwarz(0.0)
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    S, H = ctx.int1e()
    ctx.eri_store()
    kw = dict(conv=1e-10, conv_rms=True, diis=8)
    a = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, **kw)
    b = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, purify=True, **kw)
    assert ctx.stat("eig_early") == 1
    assert abs(a.energy - b.energy) < 1e-10
    assert np.max(np.abs(np.asarray(a.eig) - np.asarray(b.eig))) < 1e-8
    assert np.max(np.abs(a.D - b.D)) < 1e-8
    ea = ctx.mp2_rhf(a.eig, sysm.nelcA, PREC_FP64, C=a.C)["E_MP2"]
    eb = ctx.mp2_rhf(b.eig, sysm.nelcA, PREC_FP64, C=b.C)["E_MP2"]
    assert abs(ea - eb) < 1e-9, (ea, eb)
