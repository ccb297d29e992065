"""Replica path (several ranks, structures split between them) on CPU with gloo.

Two processes: each takes its share of a ragged batch (pyxtal_ff_gb300.replicas.shard),
evaluates a per-structure quantity on the host, and the gathered list must equal the
single-process one in the caller's order; the timing reduction must return the
slowest rank's value.  No GPU is involved: the data path has no collective, so the
multi-rank logic is all here.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from pyxtal_ff_gb300 import replicas


def _sizes():
    return np.random.default_rng(0).integers(1, 65, size=37)


def _per_structure(i, n):
    # a stand-in for a per-structure result: deterministic in (index, size)
    return float(np.sin(i + 1) * n)


def _worker(rank, world, port, queue):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = _sizes()
    mine = replicas.shard(sizes, rank, world)
    local = [_per_structure(int(i), int(sizes[i])) for i in mine]
    full = replicas.gather(local, mine)
    slowest = replicas.max_over_ranks(10.0 + rank)
    queue.put((rank, [int(i) for i in mine], full, slowest))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_covers_every_structure_once_and_balances_atoms():
    sizes = _sizes()
    for world in (1, 2, 3, 8):
        parts = [replicas.shard(sizes, r, world) for r in range(world)]
        allidx = np.concatenate(parts)
        assert sorted(allidx.tolist()) == list(range(len(sizes)))
        for p in parts:  # contiguous ranges
            assert len(p) == 0 or np.all(np.diff(p) == 1)
        loads = [int(sizes[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= 2 * int(sizes.max())
    with pytest.raises(ValueError):
        replicas.shard(sizes, 2, 2)


def test_two_ranks_gloo_gather_and_max():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    out = [queue.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sizes = _sizes()
    expect = [_per_structure(i, int(n)) for i, n in enumerate(sizes)]
    seen = []
    for rank, mine, full, slowest in sorted(out):
        assert full == expect
        assert slowest == 11.0
        seen += mine
    assert sorted(seen) == list(range(len(sizes)))
