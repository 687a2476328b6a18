"""The oracle against the reference's own known answers (no GPU).

* myQC's MOLDEN orbital energies and orbitals (examples/Be, O/singlet, NO)
  -- parity pins;
* Ftab, a known-answer table: decoded values equal the exact Boys function
  except for the four corrupted entries the reference ships;
* CFOUR energies beside the examples -- loose sanity pins (true pi, exact
  Boys, renormalised contractions in CFOUR);
* the tight oracle's Boys function against scipy's confluent hypergeometric.
"""
import json

import numpy as np
import pytest

import oracle as O
from conftest import golden, molden_orbital_errors, molden_text_of, read_molden

PINS = json.load(open(golden("reference_pins.json")))


def _run(name, ftab, basis_text, mode=0, conv_exp=None):
    return O.run_job(open(golden("zmat", name + ".ZMAT")).read(), basis_text, ftab, mode, conv_exp)


@pytest.mark.parametrize("name,tol", [("Be", 1e-8), ("O_singlet", 1e-8), ("NO", 1e-7)])
def test_molden_orbital_energies(ftab, basis_text, name, tol):
    r = _run(name, ftab, basis_text)
    p = PINS["molden"][name]
    eig = r["scf"].eig
    if p["beta"]:
        assert np.max(np.abs(eig[0] - p["alpha"])) < tol
        assert np.max(np.abs(eig[1] - p["beta"])) < tol
    else:
        assert np.max(np.abs(eig - p["alpha"])) < tol


@pytest.mark.parametrize("name,tol_e,tol_p", [("Be", 1e-8, 1e-9), ("O_singlet", 1e-8, 1e-9), ("NO", 1e-7, 1e-6)])
def test_molden_orbitals(ftab, basis_text, name, tol_e, tol_p):
    """The oracle's orbitals against the reference's MOLDEN file: energies,
    occupations and the projector onto every set of degenerate orbitals (up
    to a common rotation of the p functions, which nothing fixes for an atom
    or a linear molecule).  The NO run converges to 1e-7 like the
    reference's, so its orbitals agree to that order."""
    r = _run(name, ftab, basis_text)
    _, ref = read_molden(open(golden("molden", name + ".MOLDEN")).read())
    _, ours = read_molden(molden_text_of(r["mol"], r["scf"].eig, r["scf"].C, r["mol"].options[3] == 1))
    de, occ_ok, dp = molden_orbital_errors(ours, ref, r["basis"].basinfo)
    assert de < tol_e and occ_ok and dp < tol_p, (de, occ_ok, dp)


def test_ftab_known_answers(ftab):
    sp = pytest.importorskip("scipy.special")
    T = np.arange(121) / 10.0
    exact = np.array([[sp.hyp1f1(m + 0.5, m + 1.5, -t) / (2 * m + 1) for t in T] for m in range(23)]).T
    err = np.abs(ftab.reshape(23, 121).T - exact)
    bad = sorted((round(T[i], 1), m) for i, m in zip(*np.nonzero(err > 1e-8)))
    assert bad == [(3.6, 2), (7.4, 11), (8.4, 7), (9.4, 0)]
    # every other entry carries the table's ~10 printed digits (worst 5.7e-10 at T=1.6, m=0)
    assert np.max(np.where(err > 1e-8, 0, err)) < 1e-9


def test_tight_boys(ftab):
    sp = pytest.importorskip("scipy.special")
    for T in (0.0, 1e-3, 0.7, 5.55, 11.9, 12.0, 25.0, 35.9, 36.1, 80.0):
        F = O.boys(T, 12, ftab, mode=1)
        ex = np.array([sp.hyp1f1(m + 0.5, m + 1.5, -T) / (2 * m + 1) for m in range(13)])
        assert np.max(np.abs(F - ex) / ex) < 5e-14


@pytest.mark.parametrize("name,tol_scf,tol_mp2", [("CO2", 1e-4, 2e-6), ("HeH", 1e-6, None), ("OH", 2e-5, None)])
def test_cfour_sanity(ftab, basis_text, name, tol_scf, tol_mp2):
    r = _run(name, ftab, basis_text, conv_exp=10)
    c = PINS["cfour"][name]
    assert abs(r["scf"].energy - c["E_SCF"]) < tol_scf
    if tol_mp2:
        assert abs(r["mp2"]["E_MP2"] - c["E2(TOT)"]) < tol_mp2


def test_xx_symmetry_and_conventions(ftab, basis_text):
    """XX carries all 8 permutations; G from RHFI2G's formula equals J - K/2."""
    r = _run("HF", ftab, basis_text, conv_exp=8)
    XX = r["XX"]
    for perm in [(1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1), (3, 2, 1, 0)]:
        assert np.array_equal(XX, XX.transpose(perm))
    D = r["scf"].D
    J = np.einsum("ijkl,kl->ij", XX, D)
    K = np.einsum("ikjl,kl->ij", XX, D)
    assert np.allclose(O.fock_rhf(XX, D), J - 0.5 * K, atol=1e-12)


def test_mp2_sum_identity(ftab, basis_text):
    """E(MBPT2) = 2 E(AA) + E(AB) equals the closed-shell formula."""
    r = _run("CO2", ftab, basis_text, conv_exp=9)
    res, XX, no = r["scf"], r["XX"], r["mol"].nelcA
    C, e = res.C, res.eig
    Om = O.ao2mo(XX, C[:, :no], C[:, no:], C[:, :no], C[:, no:])
    ref = np.einsum("ua,vb,lc,sd,uvls->abcd", C[:, :no], C[:, no:], C[:, :no], C[:, no:], XX)
    assert np.allclose(Om, ref, atol=1e-12)
    D = e[:no, None, None, None] - e[None, no:, None, None] + e[None, None, :no, None] - e[None, None, None, no:]
    E = np.sum(Om * (2 * Om - Om.transpose(0, 3, 2, 1)) / D)
    assert abs(E - r["mp2"]["E_MP2"]) < 1e-12


def test_uhf_restatements_reduce_to_rhf(ftab, basis_text):
    """Closed-shell limit of the UHF restatements: UHFI2G with Da = Db = D/2
    gives RHFI2G's G for both spins, and mp2_uhf with identical spin blocks
    gives mp2_rhf's E(MBPT2) (E(AA) = E(BB), both equal to mp2_rhf's E(AA))."""
    r = _run("CO2", ftab, basis_text, conv_exp=9)
    res, XX, no = r["scf"], r["XX"], r["mol"].nelcA
    D = res.D
    Ga, Gb = O.fock_uhf(XX, 0.5 * D, 0.5 * D)
    G = O.fock_rhf(XX, D)
    assert np.allclose(Ga, G, atol=1e-12) and np.allclose(Gb, G, atol=1e-12)
    C, e = res.C, res.eig
    Om = O.ao2mo(XX, C[:, :no], C[:, no:], C[:, :no], C[:, no:])
    rh = O.mp2_rhf(e, Om)
    uh = O.mp2_uhf(e, e, Om, Om, Om)
    assert abs(uh["E_AA"] - uh["E_BB"]) < 1e-15
    assert abs(uh["E_AA"] - rh["E_AA"]) < 1e-13 and abs(uh["E_AB"] - rh["E_AB"]) < 1e-13
    assert abs(uh["E_MP2"] - rh["E_MP2"]) < 1e-12


def test_mlp_oracle_gradient_finite_differences():
    """The MLP oracle's analytic gradient (float64, no BF16 rounding) against
    central differences."""
    import mlp_ref as M
    dims = (16, 12, 12, 5)
    p = M.init_params(dims, 3)
    rng = np.random.default_rng(4)
    X = rng.standard_normal((40, dims[0]))
    T = rng.standard_normal((40, dims[3]))
    Wl = rng.random((40, dims[3]))
    _, g = M.loss_grad(p, dims, X, T, Wl, bf=False)
    idx = rng.choice(len(p), 30, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = M.loss_grad(p + e, dims, X, T, Wl, bf=False)
        lm, _ = M.loss_grad(p - e, dims, X, T, Wl, bf=False)
        assert abs((lp - lm) / (2 * h) - g[i]) < 1e-6 * max(1.0, abs(g[i]))


def test_bf16_rounding():
    import mlp_ref as M
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 0.0])
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway between 1 and 1 + 2^-7: ties to even
    assert r[2] == 1.0 + 2 ** -7  # 1.5 BF16 ulp above 1 rounds up to the even neighbour
    assert abs(r[3] + 3.140625) < 1e-12 and r[4] == 0.0


def test_cis_records_layout(ftab, basis_text):
    """The oracle's UHF CIS integral files (slow_ao2mo_CIS_UHF) on the reference's
    OH example: record counts and lengths per file, (ai|jb) symmetric under
    (ai) <-> (jb) in the same-spin files, and the ajbi records equal to
    (ab|ji) assembled from the oracle's own transform."""
    zt = open(golden("zmat", "OH.ZMAT")).read()
    ref = O.run_job(zt, basis_text, ftab, 0, conv_exp=8)
    mol, XX, C = ref["mol"], ref["XX"], ref["scf"].C
    n, noA, noB = XX.shape[0], mol.nelcA, mol.nelcB
    nvA, nvB = n - noA, n - noB
    r = O.cis_records(XX, C[0], C[1], noA, noB)
    shapes = {"ajib_AA": (noA * nvA, noA * nvA), "ajbi_AA": (noA * nvA, noA * nvA),
              "ajib_AB": (noB * nvB, noA * nvA), "ajib_BB": (noB * nvB, noB * nvB), "ajbi_BB": (noB * nvB, noB * nvB)}
    for name, (nrec, ln) in shapes.items():
        assert len(r[name]) == nrec and all(v.shape == (ln,) for v in r[name]), name
    for name, no, nv in (("ajib_AA", noA, nvA), ("ajib_BB", noB, nvB)):
        M = np.array(r[name]).reshape(no, nv, no, nv)        # [j, b, i, a]
        assert np.max(np.abs(M - M.transpose(2, 3, 0, 1))) < 1e-13
    vrt, occ = C[0][:, noA:], C[0][:, :noA]
    Om = O.ao2mo(XX, vrt, vrt, occ, occ)                     # Om[a, b, j, i] = (ab|ji)
    rec = r["ajbi_AA"][noA * nvA - 1]                         # j = noA-1, b = nvA-1
    assert np.allclose(rec, Om[:, nvA - 1, noA - 1, :].flatten(order="F"), rtol=0, atol=1e-15)


def test_dipole_integrals(ftab, basis_text):
    """The oracle's restatement of int1p (dipole integrals) and cphf_dipole_rhf:
    Px symmetric; moving every centre by t moves the integrals by t S exactly as
    x -> x + t does; the dipole of a neutral molecule does not depend on the
    origin; CO2 and H2 (centrosymmetric, centred by the parser) have none."""
    for name in ("HF", "CO2", "H2"):
        zt = open(golden("zmat", name + ".ZMAT")).read()
        ref = O.run_job(zt, basis_text, ftab, 0, conv_exp=10)
        mol, basis = ref["mol"], ref["basis"]
        P = O.int1p(mol, basis, 0)
        assert np.max(np.abs(P - P.transpose(0, 2, 1))) < 1e-15
        D = O.density(ref["scf"].C, mol.nelcA, 2.0)
        mu = O.dipole_moment(P, D, mol)
        t = np.array([0.3, -1.1, 0.7])
        moved = O.Molecule(atoms=mol.atoms, xyz=np.asarray(mol.xyz) + t, nelcA=mol.nelcA, nelcB=mol.nelcB,
                           options=mol.options)
        P2 = O.int1p(moved, basis, 0)
        S = ref["S"]
        for c in range(3):
            assert np.max(np.abs(P2[c] - (P[c] + t[c] * S))) < 1e-12
        assert np.max(np.abs(O.dipole_moment(P2, D, moved) - mu)) < 1e-10
        if name in ("CO2", "H2"):
            assert np.max(np.abs(mu)) < 1e-10
        else:
            assert abs(mu[2]) > 0.1
