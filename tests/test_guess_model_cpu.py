"""The committed learned-guess model on the CPU: the host restatement of the
prediction (descriptors, standardisation, assembly in myqc_gb300/guess.py) with
the network evaluated by the MLP oracle (oracle/mlp_ref.py, the device's BF16
rounding points), on water clusters outside the training seeds.  Each predicted
density passes the checks the library applies before it uses one -- electron
count tr(DS) within 0.5 of N, idempotency error ||DSD/2 - D|| / ||D|| below
0.25 -- with S from the oracle's one-electron integrals, and a tripled
density fails them."""
import os

import numpy as np
import pytest

from myqc_gb300 import guess, molecules

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODEL = os.path.join(ROOT, "myqc_gb300", "data", "guess_mlp.npz")


def _overlap(sym, xyz, basis_text):
    import oracle as O
    lines = ["CARTESIAN"] + [f"{s} {float(x)!r} {float(y)!r} {float(z)!r}" for s, (x, y, z) in zip(sym, xyz)]
    zt = "\n".join(lines + ["END", "", "CALC= SCF", "BASIS= STO-3G", "CHARGE= 0", "MULTI= 1", "REF= RHF"]) + "\n"
    mol = O.parse_zmat_text(zt)
    b = O.parse_mybasis_text(basis_text, mol.atoms)
    S, _ = O.int1e(mol, b, np.zeros(121 * 23), 1)
    return S, mol.nelcA + mol.nelcB


@pytest.mark.parametrize("k,seed", [(2, 911), (5, 912), (9, 913)])
def test_predicted_density_passes_the_checks(basis_text, k, seed):
    if not os.path.exists(MODEL):
        pytest.skip("no trained model")
    import mlp_ref as M
    z = np.load(MODEL)
    dims = tuple(int(v) for v in z["dims"])
    sym, xyz = molecules.water_cluster(k, (27.0 * k) ** (1 / 3), seed)
    atoms = np.array([8 if s == "O" else 1 for s in sym])
    pairs, feat, Q, t, mask = guess.pair_data(atoms, xyz)
    Xn = ((feat - z["mu_x"]) / z["sd_x"]).astype(np.float32)
    Yn, _ = M.forward(z["params"], dims, Xn)
    Y = (Yn * z["sd_y"][t] + z["mu_y"][t]) * mask
    D = guess.assemble(atoms, Y, pairs, Q)
    assert np.allclose(D, D.T, atol=1e-12)
    S, nelec = _overlap(sym, xyz, basis_text)
    assert D.shape == S.shape
    ok, dcount, idem = guess.check_density(D, S, nelec)
    assert ok, (k, dcount, idem)
    # and well inside them (the committed model: |dN| < 0.03, idempotency < 0.005)
    assert abs(dcount) < 0.1 and idem < 0.02, (k, dcount, idem)
    # a broken prediction (tripled) fails them
    assert not guess.check_density(3.0 * D, S, nelec)[0]
