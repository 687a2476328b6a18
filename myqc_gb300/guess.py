"""Learned initial density: per-atom-pair blocks in local frames.

The SCF's first density decides how many iterations follow.  The reference
starts from the core Hamiltonian (src/scf/scf.f90:410-512).  Here a small MLP
predicts the converged density block by block: for every pair of atoms (A, B)
within a cutoff, the n_A x n_B block D[A, B] expressed in a local frame of the
pair, from rotation-invariant descriptors of the pair's surroundings.  The
blocks are rotated back and assembled into D; a prediction that fails the
electron-count or idempotency check is replaced by the core guess, and so is
one whose SCF does not converge.  The SCF then converges to the same density
whatever the guess, so the guess changes the iteration count, not the result.

Local frame of a pair (A, B), A != B: e_z along A -> B; e_x towards the
nearest other atom to A (its component perpendicular to e_z); e_y = e_z x e_x.
For the diagonal block (A, A): e_z towards A's nearest atom, e_x from the next
one.  A block transforms as D_local = R_A^T D R_B with R = diag(1.., Q) acting
on the p functions (Q = [e_x e_y e_z]); s functions are invariant.

Descriptors of a pair (NFEAT numbers): the two elements, R, 1/R, and for each of
A and B its K_ENV nearest other atoms as (x, y, z in the pair frame, element
flag, 1/r).  Targets: the NOUT = 25 entries of the local block padded to 5 x 5
(an s-only atom uses row/column 0), standardised per block type.
"""
from __future__ import annotations

import numpy as np

K_ENV = 6
NFEAT = 4 + 2 * K_ENV * 5          # 64
NOUT = 25
CUTOFF = 8.0                      # Angstrom; blocks of farther pairs are taken as 0
BOHR = 1.8897161646320724
# block type of (Z_A, Z_B) with Z_A >= Z_B ordering: 0 heavy-heavy, 1 heavy-H, 2 H-H, 3 heavy diag, 4 H diag
NTYPES = 5


def ao_layout(atoms) -> tuple[np.ndarray, np.ndarray]:
    """First AO and number of AOs of each atom (STO-3G: H 1, C/N/O/F 5), in the
    reference's AO order (atoms in order; 1s, 2s, 2px, 2py, 2pz)."""
    nao = np.array([1 if int(z) <= 2 else 5 for z in atoms])
    return np.concatenate([[0], np.cumsum(nao)[:-1]]), nao


def _neighbour_order(xyz: np.ndarray):
    """Distances and, per atom, the other atoms nearest first.  Distances are
    compared rounded to 1e-6 A with ties broken by atom index, so the order (and
    every frame built from it) does not depend on rounding noise: rigid
    monomers have exactly equal O-H distances."""
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=-1)
    np.fill_diagonal(d, np.inf)
    key = np.round(d, 6)
    idx = np.broadcast_to(np.arange(len(xyz)), d.shape)
    order = np.stack([np.lexsort((idx[i], key[i])) for i in range(len(xyz))]) if len(xyz) else d.astype(int)
    return d, order


def _frames(xyz: np.ndarray, pairs: np.ndarray, order: np.ndarray | None = None) -> np.ndarray:
    """(npairs, 3, 3) rotation matrices, columns e_x, e_y, e_z of each pair frame."""
    if order is None:
        _, order = _neighbour_order(xyz)
    A, B = pairs[:, 0], pairs[:, 1]
    diag = A == B
    first = order[A, 0]
    ez = np.where(diag[:, None], xyz[first] - xyz[A], xyz[B] - xyz[A])
    ez /= np.linalg.norm(ez, axis=1, keepdims=True)
    # e_x: the first candidate neighbour of A (skipping B, and for a diagonal
    # block the neighbour that fixed e_z) with a perpendicular component
    ncand = min(order.shape[1], 6)
    ex = np.full((len(pairs), 3), np.nan)
    for k in range(ncand):
        c = order[A, k]
        v = xyz[c] - xyz[A]
        v = v - np.sum(v * ez, axis=1, keepdims=True) * ez
        nv = np.linalg.norm(v, axis=1)
        ok = (c != B) & ~(diag & (c == first)) & (nv > 1e-3) & np.isnan(ex[:, 0])
        ex[ok] = v[ok] / nv[ok, None]
    bad = np.isnan(ex[:, 0])
    if bad.any():  # collinear surroundings: any perpendicular axis
        t = np.where((np.abs(ez[bad, 0]) < 0.9)[:, None], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0])
        v = t - np.sum(t * ez[bad], axis=1, keepdims=True) * ez[bad]
        ex[bad] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return np.stack([ex, np.cross(ez, ex), ez], axis=2)


def pairs_of(atoms, xyz_angstrom: np.ndarray, cutoff: float = CUTOFF) -> np.ndarray:
    """Atom pairs (A, B), each unordered pair once and within the cutoff, plus
    the diagonal (A, A); the heavier element comes first."""
    atoms = np.asarray(atoms)
    xyz = np.asarray(xyz_angstrom, dtype=float)
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=-1)
    a, b = np.triu_indices(len(atoms))
    keep = (a == b) | (d[a, b] <= cutoff)
    a, b = a[keep], b[keep]
    swap = atoms[b] > atoms[a]
    return np.stack([np.where(swap, b, a), np.where(swap, a, b)], axis=1).astype(np.int64)


def block_type(za: np.ndarray, zb: np.ndarray, diag: np.ndarray) -> np.ndarray:
    ha, hb = za > 2, zb > 2
    t = np.where(ha & hb, 0, np.where(ha | hb, 1, 2))
    return np.where(diag, np.where(ha, 3, 4), t)


def descriptors(atoms, xyz_angstrom: np.ndarray, pairs: np.ndarray, Q: np.ndarray | None = None):
    """(features (npairs, NFEAT) float32, frames (npairs, 3, 3))."""
    atoms = np.asarray(atoms)
    xyz = np.asarray(xyz_angstrom, dtype=float)
    d, order = _neighbour_order(xyz)
    if Q is None:
        Q = _frames(xyz, pairs, order)
    P = len(pairs)
    f = np.zeros((P, NFEAT), dtype=np.float64)
    A, B = pairs[:, 0], pairs[:, 1]
    R = np.linalg.norm(xyz[B] - xyz[A], axis=1)
    f[:, 0] = atoms[A] > 2
    f[:, 1] = atoms[B] > 2
    f[:, 2] = R
    f[:, 3] = np.where(R > 0, 1.0 / np.maximum(R, 1e-9), 0.0)
    nn = min(order.shape[1], K_ENV + 1)
    for side, (X, other) in enumerate(((A, B), (B, A))):
        cand = order[X, :nn]                                   # (P, nn) nearest first
        valid = (cand != other[:, None]) & np.isfinite(d[X[:, None], cand])
        rank = np.cumsum(valid, axis=1) - 1                    # position among the kept ones
        keep = valid & (rank < K_ENV)
        pi, ci = np.nonzero(keep)
        c = cand[pi, ci]
        k = rank[pi, ci]
        loc = np.matmul((xyz[c] - xyz[X[pi]])[:, None, :], Q[pi])[:, 0, :]  # Q^T v
        base = 4 + side * K_ENV * 5 + k * 5
        for j in range(3):
            f[pi, base + j] = loc[:, j]
        f[pi, base + 3] = atoms[c] > 2
        f[pi, base + 4] = 1.0 / d[X[pi], c]
    return f.astype(np.float32), Q


def _rot(natoms_ao: int, Q: np.ndarray) -> np.ndarray:
    """AO rotation of one atom's functions for frame Q: identity on s, Q on p."""
    R = np.eye(natoms_ao)
    if natoms_ao == 5:
        R[2:5, 2:5] = Q
    return R


def _ao_index(atoms, pairs):
    """Padded 5 x 5 AO index grids of each pair's block and their validity."""
    first, nao = ao_layout(atoms)
    r = np.arange(5)
    a, b = pairs[:, 0], pairs[:, 1]
    ia = first[a][:, None] + r[None, :]
    ib = first[b][:, None] + r[None, :]
    va = r[None, :] < nao[a][:, None]
    vb = r[None, :] < nao[b][:, None]
    return np.where(va, ia, 0), np.where(vb, ib, 0), va, vb


def _rots(atoms, pairs, Q):
    """(npairs, 5, 5) AO rotations of A and B: identity on s, Q on p."""
    _, nao = ao_layout(atoms)
    Ra = np.broadcast_to(np.eye(5), (len(pairs), 5, 5)).copy()
    Rb = Ra.copy()
    ha = nao[pairs[:, 0]] == 5
    hb = nao[pairs[:, 1]] == 5
    Ra[ha, 2:5, 2:5] = Q[ha]
    Rb[hb, 2:5, 2:5] = Q[hb]
    return Ra, Rb


def extract_blocks(atoms, D: np.ndarray, pairs: np.ndarray, Q: np.ndarray) -> np.ndarray:
    """(npairs, NOUT) local-frame blocks of D, padded to 5 x 5 (row-major)."""
    ia, ib, va, vb = _ao_index(atoms, pairs)
    blk = D[ia[:, :, None], ib[:, None, :]] * (va[:, :, None] & vb[:, None, :])
    Ra, Rb = _rots(atoms, pairs, Q)
    out = np.matmul(np.matmul(Ra.transpose(0, 2, 1), blk), Rb)  # Ra^T blk Rb
    return out.reshape(len(pairs), NOUT)


def assemble(atoms, blocks: np.ndarray, pairs: np.ndarray, Q: np.ndarray) -> np.ndarray:
    """Density from local-frame blocks (inverse of extract_blocks); pairs
    absent from the list give zero blocks; diagonal blocks are symmetrised."""
    _, nao = ao_layout(atoms)
    n = int(nao.sum())
    ia, ib, va, vb = _ao_index(atoms, pairs)
    m = (va[:, :, None] & vb[:, None, :])
    Ra, Rb = _rots(atoms, pairs, Q)
    b5 = blocks.reshape(len(pairs), 5, 5) * m
    blk = np.matmul(np.matmul(Ra, b5), Rb.transpose(0, 2, 1))  # Ra b5 Rb^T
    diag = pairs[:, 0] == pairs[:, 1]
    blk[diag] = 0.5 * (blk[diag] + np.transpose(blk[diag], (0, 2, 1)))
    D = np.zeros((n, n))
    rows = np.broadcast_to(ia[:, :, None], blk.shape)[m]
    cols = np.broadcast_to(ib[:, None, :], blk.shape)[m]
    D[rows, cols] = blk[m]
    D[cols, rows] = blk[m]
    return D


def output_mask(atoms, pairs: np.ndarray) -> np.ndarray:
    """(npairs, NOUT) 1 where the padded 5 x 5 block holds a real entry."""
    _, nao = ao_layout(atoms)
    r = np.arange(5)
    va = r[None, :] < nao[pairs[:, 0]][:, None]
    vb = r[None, :] < nao[pairs[:, 1]][:, None]
    return (va[:, :, None] & vb[:, None, :]).reshape(len(pairs), NOUT).astype(np.float32)


def check_density(D: np.ndarray, S: np.ndarray, nelec: int, tol_count: float = 0.5, tol_idem: float = 0.25):
    """Electron count tr(DS) and idempotency ||D S D / 2 - D|| / ||D|| of a
    closed-shell guess; returns (ok, count_error, idempotency_error)."""
    cnt = float(np.trace(D @ S))
    idem = float(np.linalg.norm(0.5 * D @ S @ D - D) / max(np.linalg.norm(D), 1e-30))
    ok = np.isfinite(cnt) and abs(cnt - nelec) < tol_count and idem < tol_idem
    return ok, cnt - nelec, idem


# ---------------------------------------------------------------- model I/O and inference
def system_geometry(sysm):
    """(atoms, xyz in Angstrom) of a System (whose xyz is in bohr)."""
    return np.asarray(sysm.atoms), np.asarray(sysm.xyz, dtype=float) / BOHR


def pair_data(atoms, xyz_angstrom):
    """Pairs, descriptors, frames, block types and output masks of one geometry."""
    pairs = pairs_of(atoms, xyz_angstrom)
    feat, Q = descriptors(atoms, xyz_angstrom, pairs)
    za, zb = np.asarray(atoms)[pairs[:, 0]], np.asarray(atoms)[pairs[:, 1]]
    t = block_type(za, zb, pairs[:, 0] == pairs[:, 1])
    return pairs, feat, Q, t, output_mask(atoms, pairs)


class LearnedGuess:
    """Trained network + normalisation, evaluated in the library
    (mq_guess_predict: descriptors, forward pass and assembly on the GPU).
    The file holds params (FP32), dims, mu_x/sd_x (feature standardisation)
    and mu_y/sd_y (per block type and output entry).  `predict` is the host
    restatement of the same steps (the training set's descriptors are formed
    by it), kept for the tests that compare the two."""

    def __init__(self, ctx, path: str):
        z = np.load(path)
        self.ctx = ctx
        self.dims = tuple(int(v) for v in z["dims"])
        self.mu_x, self.sd_x = z["mu_x"], z["sd_x"]
        self.mu_y, self.sd_y = z["mu_y"], z["sd_y"]
        ctx.guess_model(self.dims, z["params"], self.mu_x, self.sd_x, self.mu_y, self.sd_y)

    def predict(self, atoms, xyz_angstrom) -> np.ndarray:
        pairs, feat, Q, t, mask = pair_data(atoms, xyz_angstrom)
        Xn = (feat - self.mu_x) / self.sd_x
        Yn = self.ctx.mlp_forward(Xn.astype(np.float32)).astype(np.float64)
        Y = (Yn * self.sd_y[t] + self.mu_y[t]) * mask
        return assemble(atoms, Y, pairs, Q)

    def predict_many(self, systems) -> list:
        """Predicted densities of many systems, on the GPU in one pass."""
        return self.ctx.guess_predict(systems)

    def guess(self, sysm, S: np.ndarray):
        """Predicted closed-shell density, or None when it fails the
        electron-count or idempotency check (the caller then uses the core
        guess)."""
        D = self.ctx.guess_predict([sysm])[0]
        ok, _, _ = check_density(D, S, sysm.nelcA + sysm.nelcB)
        return D if ok else None
