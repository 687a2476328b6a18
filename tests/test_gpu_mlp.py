"""The learned guess's network on the tensor cores against the CPU oracle
(oracle/mlp_ref.py): forward values, gradients of all six parameter blocks
(two split-K chunks of samples), one Adam step, and that training lowers the
loss on a teacher-network regression."""
import numpy as np
import pytest

import mlp_ref as M

pytestmark = pytest.mark.gpu

DIMS = (64, 256, 256, 25)


def _data(rows, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((rows, DIMS[0])).astype(np.float32)
    T = rng.standard_normal((rows, DIMS[3])).astype(np.float32)
    W = (rng.random((rows, DIMS[3])) < 0.7).astype(np.float32)
    return X, T, W


def _blocks(v):
    out, o = [], 0
    for l in range(3):
        for n in (DIMS[l + 1] * DIMS[l], DIMS[l + 1]):
            out.append(v[o:o + n])
            o += n
    return out


def test_mlp_forward_and_gradients(ctx):
    ctx.mlp_init(DIMS[0], DIMS[1], DIMS[3])
    p = M.init_params(DIMS, 1).astype(np.float32)
    ctx.mlp_set_params(p)
    assert np.array_equal(ctx.mlp_get_params(), p)
    X, T, W = _data(3000, 2)
    ref, _ = M.forward(p, DIMS, X)
    out = ctx.mlp_forward(X)
    assert np.max(np.abs(out - ref)) < 5e-3 * np.max(np.abs(ref))
    loss, g = ctx.mlp_grad(X, T, W)
    lref, gref = M.loss_grad(p, DIMS, X, T, W)
    assert abs(loss - lref) < 1e-3 * lref
    for a, b in zip(_blocks(g), _blocks(gref)):
        assert np.linalg.norm(a - b) < 2e-2 * np.linalg.norm(b) + 1e-7


def test_mlp_adam_step_and_training(ctx):
    ctx.mlp_init(DIMS[0], DIMS[1], DIMS[3])
    p0 = M.init_params(DIMS, 5).astype(np.float32)
    ctx.mlp_set_params(p0)
    X, T, W = _data(1024, 6)
    # one epoch of one full batch = one Adam step on the full-batch gradient
    _, g = ctx.mlp_grad(X, T, W)
    ctx.mlp_set_data(X, T, W)
    ctx.mlp_train_epoch(1024, 1e-3, 0)
    p1 = ctx.mlp_get_params()
    pr, _, _ = M.adam_step(p0.astype(np.float64), 0.0, 0.0, g.astype(np.float64), 1, 1e-3)
    assert np.max(np.abs(p1 - pr)) < 1e-5 + 1e-3 * np.max(np.abs(pr - p0))
    # teacher regression: the loss falls
    teacher = M.init_params(DIMS, 9)
    Xt, _, _ = _data(16384, 10)
    Tt, _ = M.forward(teacher, DIMS, Xt)
    Wt = np.ones_like(Tt, dtype=np.float32)
    ctx.mlp_set_params(M.init_params(DIMS, 11).astype(np.float32))
    ctx.mlp_set_data(Xt, Tt.astype(np.float32), Wt)
    losses = [ctx.mlp_train_epoch(1024, 1e-3, e) for e in range(12)]
    assert losses[-1] < 0.3 * losses[0], losses
