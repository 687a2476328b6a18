"""CPU oracle of the learned guess's network (mlp.cu).

TEST INFRASTRUCTURE ONLY: the parity checker for libmyqc's MLP kernels; only
tests/ import it.  It restates the network in float64 NumPy: 3 layers
nin -> width -> width -> nout, SiLU, weighted squared loss, with the GPU's BF16
rounding points emulated (round to nearest even) so that the device's forward
values and gradients can be compared to it:
    x, W are BF16; z1 = x W1^T + b1; y1 = bf16(SiLU(z1)); z2, y2 likewise;
    out = y2 W3^T + b3; dy3 = bf16(2 w (out - t) / sum w);
    dz2 = bf16((dy3 W3) SiLU'(z2)); dz1 = bf16((dz2 W2) SiLU'(z1));
    gW3 = dy3^T y2, gW2 = dz2^T y1, gW1 = dz1^T x, gb = column sums.
With bf16=False every rounding is skipped: the plain float64 network, whose
analytic gradient is checked against finite differences.
Adam (Kingma and Ba, 2015) is restated for the optimiser test.
"""
from __future__ import annotations

import numpy as np


def bf16(a):
    """Round float values to BF16 (nearest, ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def unpack(params, dims):
    out, o = [], 0
    for l in range(3):
        nw = dims[l + 1] * dims[l]
        W = np.asarray(params[o:o + nw], dtype=np.float64).reshape(dims[l + 1], dims[l])
        o += nw
        b = np.asarray(params[o:o + dims[l + 1]], dtype=np.float64)
        o += dims[l + 1]
        out.append((W, b))
    return out


def pack(grads):
    return np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])


def forward(params, dims, X, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    (W1, b1), (W2, b2), (W3, b3) = unpack(params, dims)
    x = r(X)
    z1 = x @ r(W1).T + b1
    y1 = r(silu(z1))
    z2 = y1 @ r(W2).T + b2
    y2 = r(silu(z2))
    out = y2 @ r(W3).T + b3
    return out, (x, z1, y1, z2, y2)


def loss_grad(params, dims, X, T, Wl, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    (W1, b1), (W2, b2), (W3, b3) = unpack(params, dims)
    out, (x, z1, y1, z2, y2) = forward(params, dims, X, bf)
    wsum = float(np.sum(Wl))
    loss = float(np.sum(Wl * (out - T) ** 2) / wsum)
    dy3 = r(2.0 * Wl * (out - T) / wsum)
    dz2 = r((dy3 @ r(W3)) * dsilu(z2))
    dz1 = r((dz2 @ r(W2)) * dsilu(z1))
    grads = [(dz1.T @ x, dz1.sum(0)), (dz2.T @ y1, dz2.sum(0)), (dy3.T @ y2, dy3.sum(0))]
    return loss, pack(grads)


def adam_step(params, m, v, g, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def init_params(dims, seed=0):
    """Scaled normal initialisation (fan-in), zero biases."""
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(3):
        W = rng.standard_normal((dims[l + 1], dims[l])) * np.sqrt(1.0 / dims[l])
        parts.append(np.concatenate([W.ravel(), np.zeros(dims[l + 1])]))
    return np.concatenate(parts)
