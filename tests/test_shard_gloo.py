"""Group sharding across two ranks with the gloo backend on CPU: LPT
assignment covers every group once and balances the estimated cost; the
counts gather and the max-over-ranks timing reduction work across ranks."""
import os
import sys

import numpy as np
import torch.multiprocessing as mp

from conftest import ROOT


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import load_pkg
    load_pkg()
    from mpi_rockstar_gb300 import shard
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = np.random.default_rng(1).integers(10, 20000, size=300)
    owner = shard.lpt_partition(sizes, world)
    mine = int((owner == rank).sum())
    counts = shard.gather_counts(mine)
    t = shard.max_over_ranks(1.5 + rank)
    q.put((rank, counts, t, owner.tolist()))
    dist.destroy_process_group()


def test_two_rank_sharding():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29511
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
    res.sort()
    assert res[0][1] == res[1][1] and sum(res[0][1]) == 300
    assert res[0][2] == res[1][2] == 2.5
    assert res[0][3] == res[1][3]


def test_lpt_balance():
    import importlib
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import load_pkg
    load_pkg()
    from mpi_rockstar_gb300 import shard
    sizes = np.random.default_rng(2).pareto(0.9, size=5000) * 20 + 20
    owner = shard.lpt_partition(sizes, 8)
    load = np.bincount(owner, weights=shard.group_cost(sizes), minlength=8)
    assert load.max() <= 1.05 * load.mean() + shard.group_cost(sizes).max()
