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


def test_native_prediction_matches_host(ctx, basis_text):
    """The library's predictor (descriptors, forward pass and assembly on the
    GPU, mq_guess_predict) against the host restatement the training set was
    built with, fed through the same network: the same densities, for clusters
    inside and outside the training range, one call for all of them."""
    if not os.path.exists(MODEL):
        pytest.skip("no trained model")
    lg = guess.LearnedGuess(ctx, MODEL)
    systems = [s for _, s, _ in _clusters(basis_text)]
    got = lg.predict_many(systems)
    for s, D in zip(systems, got):
        ref = lg.predict(*guess.system_geometry(s))
        assert D.shape == ref.shape
        assert np.max(np.abs(D - ref)) < 1e-6 * max(1.0, np.max(np.abs(ref))), len(s.atoms)


def test_batched_guess_checks_and_iterations(ctx, basis_text):
    """Held-out clusters ((H2O)_2..16, seeds outside the training set) solved
    by the batched SCF from the core guess and from the predicted densities:
    the batch's own checks accept every prediction, the converged energies
    agree to 1e-9 Eh, the learned guess takes at least 1.4x fewer iterations on
    average; a broken prediction (the density tripled) fails the electron-count
    check and the core guess is used, with the core guess's iterations."""
    if not os.path.exists(MODEL):
        pytest.skip("no trained model")
    from myqc_gb300 import train_guess
    lg = guess.LearnedGuess(ctx, MODEL)
    systems = train_guess.geometries(64, 424242)
    ctx.basis_library(basis_text)

    def run(guesses):
        ctx.batch_clear()
        for s in systems:
            ctx.batch_add_atoms(s)
        out = ctx.batch_scf(D_guess=guesses, **train_guess.SCF)
        return out, ctx.stat("guesses_taken")

    core, _ = run(None)
    preds = lg.predict_many(systems)
    learned, taken = run(preds)
    broken, taken_broken = run([3.0 * D for D in preds])
    ctx.batch_clear()
    assert taken == len(systems) and taken_broken == 0
    assert core["converged"].all() and learned["converged"].all()
    assert np.max(np.abs(learned["energy"] - core["energy"])) < 1e-9
    assert np.array_equal(broken["iterations"], core["iterations"])
    ratio = np.mean(core["iterations"]) / np.mean(learned["iterations"])
    assert ratio >= 1.4, ratio
