"""The learned initial density (myqc_gb300/data/guess_mlp.npz, trained by
myqc_gb300/train_guess.py on batched-SCF densities of (H2O)_2..16) against the
core-Hamiltonian guess on held-out clusters: fewer SCF iterations to the same
converged energy (1e-9 Eh), and a failing prediction falls back to the core
guess."""
import os

import numpy as np
import pytest

from myqc_gb300 import MODE_TIGHT, formats, guess, molecules

pytestmark = pytest.mark.gpu

MODEL = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "myqc_gb300", "data",
                     "guess_mlp.npz")
KW = dict(conv=1e-10, conv_rms=True, diis=8, max_iter=200)


def _clusters(basis_text):
    out = []
    for k, seed in ((4, 901), (9, 902), (16, 903), (24, 904)):  # (H2O)24 is larger than any training cluster
        sysm = molecules.water_cluster_system(k, (27.0 * k) ** (1 / 3), seed)
        out.append((k, sysm, formats.parse_mybasis_text(basis_text, sysm.atoms)))
    return out


def test_learned_guess_cuts_iterations(ctx, basis_text):
    if not os.path.exists(MODEL):
        pytest.skip("no trained model")
    lg = guess.LearnedGuess(ctx, MODEL)
    core_it, learned_it = [], []
    for k, sysm, basis in _clusters(basis_text):
        ctx.set_system(sysm, basis, None, MODE_TIGHT)
        S, H = ctx.int1e()
        ctx.eri_store()
        a = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, **KW)
        D0 = lg.guess(sysm, S)
        assert D0 is not None, k
        b = ctx.scf(S, H, sysm.nelcA, sysm.nelcB, D_guess=D0, **KW)
        assert abs(a.energy - b.energy) < 1e-9, (k, a.energy, b.energy)
        core_it.append(a.iterations)
        learned_it.append(b.iterations)
    assert np.mean(learned_it) < np.mean(core_it), (core_it, learned_it)


def test_failed_prediction_falls_back(ctx, basis_text):
    if not os.path.exists(MODEL):
        pytest.skip("no trained model")
    lg = guess.LearnedGuess(ctx, MODEL)
    ctx.mlp_set_params(np.zeros(ctx.mlp_param_count(), dtype=np.float32) + 3.0)  # a broken network
    k, sysm, basis = _clusters(basis_text)[0]
    ctx.set_system(sysm, basis, None, MODE_TIGHT)
    S, _ = ctx.int1e()
    assert lg.guess(sysm, S) is None
