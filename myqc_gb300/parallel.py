"""Replicas across GPUs: independent molecules shard over ranks.

The path has no exchange step between molecules: each rank solves its own
share of a batch on its own GPU, with no collective on the data path, and the
results are gathered once at the end.  A single
molecule is not split across GPUs.

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
