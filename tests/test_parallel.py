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
