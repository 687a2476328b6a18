"""Replica sharding across ranks, on CPU: world_size 2 over gloo (127.0.0.1)."""
import os
import socket

import numpy as np
import pytest

from myqc_gb300 import parallel


def test_shard_balances_and_covers():
    rng = np.random.default_rng(0)
    costs = rng.integers(1, 100, size=57).astype(float) ** 2
    for world in (1, 2, 3, 8):
        parts = parallel.shard(costs, world)
        assert len(parts) == world
        flat = [i for p in parts for i in p]
        assert flat == list(range(len(costs)))
        if world > 1:
            loads = [costs[p].sum() for p in parts]
            assert max(loads) - min(loads) <= costs.max() * 2


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = [float(k % 7 + 1) ** 4 for k in range(23)]
    mine = parallel.shard(costs, world)[rank]
    results = [(k, k * k + 0.5) for k in mine]  # stands in for a rank's SCF results
    out = parallel.gather(results, mine, rank, world, len(costs))
    if rank == 0:
        q.put(out)
    dist.barrier()
    dist.destroy_process_group()


def test_gather_two_ranks_gloo():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out == [(k, k * k + 0.5) for k in range(23)]


# ---- one molecule split over ranks: the host protocol, with the oracle as each rank's Fock build
_CO2 = "CARTESIAN\nC 0.00 0.00 0.00\nO 0.00 0.00 -1.16\nO 0.00 0.00 1.16\nEND\n\nCALC= SCF\nBASIS= STO-3G\n" \
       "CHARGE= 0\nMULTI= 1\nREF= RHF\n"


class _OracleShare:
    """Stands in for a rank's GPU context: its Fock build digests only its share
    of the integral array (slabs (i, j) with i + n j = part mod nparts); G is
    linear in the integrals, so the shares' G matrices sum to the full G."""

    def __init__(self, XX):
        self.XX, self.part, self.nparts = XX, 0, 1

    def set_partition(self, part, nparts):
        self.part, self.nparts = part, nparts

    def fock(self, D, direct=True):
        import oracle as O
        n = D.shape[0]
        ij = (np.arange(n)[:, None] + n * np.arange(n)[None, :]) % self.nparts == self.part
        return O.fock_rhf(self.XX * ij[:, :, None, None], D)


def _co2_oracle():
    import oracle as O
    root = os.path.dirname(os.path.abspath(__file__))
    btext = open(os.path.join(root, "golden", "mybasis")).read()
    mol = O.parse_zmat_text(_CO2)
    b = O.parse_mybasis_text(btext, mol.atoms)
    ft = np.zeros(121 * 23)
    S, H = O.int1e(mol, b, ft, 1)
    return mol, S, H, O.int2e(mol, b, ft, 1), O.nuclear_repulsion(mol)


def _split_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mol, S, H, XX, enuc = _co2_oracle()
    E, e, C, D, it = parallel.scf_split(_OracleShare(XX), S, H, mol.nelcA, enuc, rank, world)
    q.put((rank, E, it))
    dist.barrier()
    dist.destroy_process_group()


def test_split_molecule_two_ranks_gloo():
    """Two ranks, each digesting half of the integrals, joined by one all-reduce
    of G per iteration, converge to the one-rank SCF (same iterations, energy
    within 1e-10 Eh), and that is the oracle's own Roothaan fixed point."""
    pytest.importorskip("torch")
    import multiprocessing as mp
    import oracle as O
    mol, S, H, XX, enuc = _co2_oracle()
    E1, e1, C1, D1, it1 = parallel.scf_split(_OracleShare(XX), S, H, mol.nelcA, enuc, 0, 1)
    F = H + O.fock_rhf(XX, D1)
    assert abs(0.5 * float(np.sum(D1 * (F + H))) + enuc - E1) < 1e-12
    ref = O.scf(mol, S, H, XX, conv_exp=10)
    if ref.converged:
        assert abs(ref.energy - E1) < 1e-9
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_split_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, E, it in out:
        assert abs(E - E1) < 1e-10 and it == it1, (rank, E, E1, it, it1)
