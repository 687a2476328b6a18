"""Host side of the learned density guess: pair frames, descriptors, block
extraction and assembly (no GPU)."""
import numpy as np

from myqc_gb300 import guess, molecules


def _cluster(k=3, seed=2):
    sym, xyz = molecules.water_cluster(k, (27.0 * k) ** (1 / 3) + 1.0, seed)
    atoms = np.array([8 if s == "O" else 1 for s in sym])
    return atoms, xyz


def _rand_density(atoms, rng):
    _, nao = guess.ao_layout(atoms)
    n = int(nao.sum())
    D = rng.standard_normal((n, n))
    return D + D.T


def _ao_rotation(atoms, R):
    first, nao = guess.ao_layout(atoms)
    n = int(nao.sum())
    U = np.eye(n)
    for a in range(len(atoms)):
        if nao[a] == 5:
            U[first[a] + 2:first[a] + 5, first[a] + 2:first[a] + 5] = R
    return U


def test_extract_assemble_round_trip():
    atoms, xyz = _cluster()
    rng = np.random.default_rng(0)
    D = _rand_density(atoms, rng)
    pairs = guess.pairs_of(atoms, xyz, cutoff=1e9)
    feat, Q = guess.descriptors(atoms, xyz, pairs)
    assert feat.shape == (len(pairs), guess.NFEAT)
    blocks = guess.extract_blocks(atoms, D, pairs, Q)
    assert np.allclose(guess.assemble(atoms, blocks, pairs, Q), D, atol=1e-12)
    # every frame is a proper rotation
    for q in Q:
        assert np.allclose(q.T @ q, np.eye(3), atol=1e-12) and abs(np.linalg.det(q) - 1) < 1e-12


def test_rotation_invariance():
    atoms, xyz = _cluster(4, 7)
    rng = np.random.default_rng(1)
    D = _rand_density(atoms, rng)
    pairs = guess.pairs_of(atoms, xyz)
    f1, Q1 = guess.descriptors(atoms, xyz, pairs)
    b1 = guess.extract_blocks(atoms, D, pairs, Q1)
    R = molecules.random_rotation(rng)
    xyz2 = xyz @ R.T + np.array([1.0, -2.0, 0.5])
    U = _ao_rotation(atoms, R)
    D2 = U @ D @ U.T
    f2, Q2 = guess.descriptors(atoms, xyz2, pairs)
    b2 = guess.extract_blocks(atoms, D2, pairs, Q2)
    assert np.allclose(f1, f2, atol=1e-5)
    assert np.allclose(b1, b2, atol=1e-10)


def test_masks_and_types():
    atoms, xyz = _cluster(2, 1)
    pairs = guess.pairs_of(atoms, xyz)
    m = guess.output_mask(atoms, pairs)
    za, zb = atoms[pairs[:, 0]], atoms[pairs[:, 1]]
    t = guess.block_type(za, zb, pairs[:, 0] == pairs[:, 1])
    expect = {0: 25, 1: 5, 2: 1, 3: 25, 4: 1}
    for p in range(len(pairs)):
        assert m[p].sum() == expect[int(t[p])]
    assert (za >= zb).all()
