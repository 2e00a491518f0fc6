"""Mesh sharding across ranks: a partition, balanced, identical on every rank (gloo, 2 ranks)."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from bvh_gb300 import meshgen, shard


def test_assign_is_a_balanced_partition():
    counts = meshgen.batch_counts(4096, 64, 262144, seed=4)
    for ws in (1, 2, 3, 8):
        parts = shard.assign(counts, ws)
        allm = np.sort(np.concatenate(parts))
        assert np.array_equal(allm, np.arange(len(counts)))
        loads = np.array([counts[p].sum() for p in parts])
        assert loads.max() - loads.min() <= counts.max()


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    counts = meshgen.batch_counts(500, 64, 5000, seed=9)
    mine = shard.assign(counts, world)[rank]
    # every rank derives the same partition on its own; check it through one all_gather
    import torch
    t = torch.zeros(len(counts), dtype=torch.int64)
    t[torch.from_numpy(mine)] = rank + 1
    gathered = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(gathered, t)
    owners = sum(gathered)
    ok = bool((owners > 0).all()) and bool((torch.stack(gathered).gt(0).sum(0) == 1).all())
    offs = shard.shard_offsets(counts, mine)
    ok = ok and int(offs[-1]) == int(counts[mine].sum())
    out[rank] = 1 if ok else 0
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_partition():
    ctx = mp.get_context("spawn")
    out = ctx.Array("i", [0, 0])
    port = 29000 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert list(out) == [1, 1]


def _worker_shares(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    ok = True
    # a serving stream: every request served by exactly one rank, loads balanced by size
    g = np.random.default_rng(7)
    sizes = np.exp(g.uniform(np.log(1000), np.log(2e6), 32)).astype(np.int64)
    picks = g.integers(0, 32, 4000)
    mine = shard.stream_share(sizes[picks], world, rank)
    t = torch.zeros(4000, dtype=torch.int64)
    t[torch.from_numpy(mine)] = 1
    dist.all_reduce(t)
    ok = ok and bool((t == 1).all())
    # a rank's share of a batch, generated alone, equals those meshes generated together
    counts = meshgen.batch_counts(64 * world, 64, 3000, seed=4)
    part = shard.assign(counts, world)[rank]
    m, offs = meshgen.batch_subset(counts, part, seed=5)
    whole, woffs = meshgen.batch_subset(counts, np.arange(len(counts)), seed=5)
    for j, k in enumerate(part):
        for a, b in zip(m.arrays(), whole.arrays()):
            ok = ok and np.array_equal(a[offs[j]:offs[j + 1]], b[woffs[k]:woffs[k + 1]])
    ok = ok and int(offs[-1]) == int(counts[part].sum())
    out[rank] = 1 if ok else 0
    dist.destroy_process_group()


def test_two_gloo_ranks_share_the_stream_and_the_batch():
    ctx = mp.get_context("spawn")
    out = ctx.Array("i", [0, 0])
    port = 30000 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker_shares, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert list(out) == [1, 1]
