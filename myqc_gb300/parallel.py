"""Several GPUs, one process each: replicas of a batch, or one molecule split.

Replicas: the path has no exchange step between molecules, so each rank
solves its own share of a batch on its own GPU, with no collective on the data
path, and the results are gathered once at the end.

One large molecule: every rank keeps the shell quartets whose bra shell pair
index falls to it (mq_set_partition, quartet store or direct builds), its
Fock build returns that share's part of G, and one all-reduce (sum) of the
n x n G per iteration gives every rank the full G (`fock_allreduce`); the rest
of the iteration (DIIS, the eigensolve, the density) is cheap and repeated on
every rank (`scf_split`).  This is the operation of RHFI2G
(src/I2G/RHFI2G.f90:80-90) split over the integral list.

`shard` assigns molecules to ranks in contiguous blocks balanced by cost (the
number of basis functions to the fourth power, the integral and Fock work);
`gather` restores the original order on rank 0 through torch.distributed
(gloo on CPU, NCCL on GPUs).  `solve_sharded` is the batched SCF on each
rank's share.
"""
from __future__ import annotations

import numpy as np


def cost(sysm) -> float:
    n = sum(1 if int(z) <= 2 else 5 for z in sysm.atoms)
    return float(n) ** 4


def shard(costs, world: int):
    """Contiguous blocks of indices, one per rank, with near-equal total cost
    (greedy cut of the cumulative cost at the rank boundaries)."""
    costs = np.asarray(costs, dtype=float)
    if world <= 1 or len(costs) == 0:
        return [list(range(len(costs)))] + [[] for _ in range(max(world, 1) - 1)]
    cum = np.cumsum(costs)
    total = cum[-1]
    cuts = [int(np.searchsorted(cum, total * r / world, side="left")) for r in range(1, world)]
    bounds = [0] + cuts + [len(costs)]
    return [list(range(bounds[r], bounds[r + 1])) for r in range(world)]


def gather(local_results, local_indices, rank: int, world: int, total: int):
    """Results of all ranks in the original order (rank 0; None elsewhere)."""
    if world <= 1:
        return list(local_results)
    import torch.distributed as dist
    objs = [None] * world if rank == 0 else None
    dist.gather_object((list(local_indices), list(local_results)), objs, dst=0)
    if rank != 0:
        return None
    out = [None] * total
    for idx, res in objs:
        for i, r in zip(idx, res):
            out[i] = r
    return out


def solve_sharded(ctx, systems, bases, rank: int, world: int, **scf_kw):
    """Batched SCF of this rank's share; returns (indices, per-molecule
    (energy, iterations, converged))."""
    parts = shard([cost(s) for s in systems], world)
    mine = parts[rank]
    ctx.batch_clear()
    for i in mine:
        ctx.batch_add(systems[i], bases[i])
    if not mine:
        return mine, []
    out = ctx.batch_scf(**scf_kw)
    res = [(float(out["energy"][k]), int(out["iterations"][k]), bool(out["converged"][k])) for k in range(len(mine))]
    return mine, res


def nuclear_repulsion(sysm) -> float:
    """E_nuc = sum_{A<B} Z_A Z_B / R_AB (getEnr, src/scf/scf.f90:1122-1152), bohr."""
    Z = np.asarray(sysm.atoms, dtype=float)
    x = np.asarray(sysm.xyz, dtype=float).reshape(-1, 3)
    e = 0.0
    for a in range(len(Z)):
        for b in range(a):
            e += Z[a] * Z[b] / float(np.linalg.norm(x[a] - x[b]))
    return e


def allreduce_sum(A: np.ndarray) -> np.ndarray:
    """Sum of a host array over the ranks of the default process group (the
    array itself without one).  NCCL reduces device tensors, gloo host ones."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return A
    import torch
    t = torch.from_numpy(np.ascontiguousarray(A))
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def fock_allreduce(ctx, D: np.ndarray, direct: bool = True) -> np.ndarray:
    """The full RHF G of the molecule: this rank's share (its partition of the
    shell quartets, set with ctx.set_partition), summed over the ranks."""
    return allreduce_sum(ctx.fock(D, direct=direct))


def scf_split(ctx, S, H, nocc: int, enuc: float, rank: int, world: int, conv: float = 1e-10, diis: int = 8,
              max_iter: int = 100, direct: bool = True):
    """RHF SCF of one molecule split over `world` ranks: each rank's Fock
    build covers its share of the shell quartets and one all-reduce of G per
    iteration joins them; DIIS(diis) on F with the commutator error FDS - SDF,
    eigenvectors of F C = S C e, D = 2 C_occ C_occ^T, until the RMS density
    change is below conv.  Returns (energy, eigenvalues, C, D, iterations)."""
    from scipy.linalg import eigh, solve
    ctx.set_partition(rank, world)
    try:
        e, C = eigh(H, S)
        D = 2.0 * C[:, :nocc] @ C[:, :nocc].T
        Fs, Es = [], []
        E = 0.0
        for it in range(1, max_iter + 1):
            G = fock_allreduce(ctx, D, direct=direct)
            F = H + G
            E = 0.5 * float(np.sum(D * (F + H))) + enuc
            if diis > 0:
                err = F @ D @ S - S @ D @ F
                Fs.append(F)
                Es.append(err)
                Fs, Es = Fs[-diis:], Es[-diis:]
                m = len(Fs)
                if m >= 2:
                    B = -np.ones((m + 1, m + 1))
                    B[m, m] = 0.0
                    for i in range(m):
                        for j in range(m):
                            B[i, j] = float(np.sum(Es[i] * Es[j]))
                    rhs = np.zeros(m + 1)
                    rhs[m] = -1.0
                    cvec = solve(B, rhs)[:m]
                    F = sum(ci * Fi for ci, Fi in zip(cvec, Fs))
            e, C = eigh(F, S)
            Dn = 2.0 * C[:, :nocc] @ C[:, :nocc].T
            rms = float(np.sqrt(np.mean((Dn - D) ** 2)))
            if rms < conv:
                return E, e, C, D, it
            D = Dn
        raise RuntimeError("split SCF did not converge")
    finally:
        ctx.set_partition(0, 1)
