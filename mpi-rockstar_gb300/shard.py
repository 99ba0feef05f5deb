"""Group-level sharding across ranks (one process per GPU).

After the 3D FOF the groups are independent units -- the reference hands them
to OpenMP threads (src/mpi_main.cpp:1363-1389).  Across GPUs they are
assigned by longest-processing-time bin packing on an n log n cost estimate;
each rank runs find_subs on its share with no data-path collective, and the
halo catalogues are gathered once at the end.
"""
import numpy as np


def group_cost(sizes):
    s = np.asarray(sizes, np.float64)
    return s * np.log2(s + 2.0)


def lpt_partition(sizes, nranks):
    """Rank of every group: largest estimated cost first, to the least loaded
    rank (ties to the lower rank).  Deterministic."""
    cost = group_cost(sizes)
    order = np.lexsort((np.arange(len(cost)), -cost))
    load = np.zeros(nranks)
    owner = np.empty(len(cost), np.int64)
    for g in order:
        r = int(np.argmin(load))
        owner[g] = r
        load[r] += cost[g]
    return owner


def gather_counts(local_count, group=None):
    """All ranks' halo counts (torch.distributed, any backend)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([local_count], dtype=torch.int64)
    out = [torch.zeros(1, dtype=torch.int64) for _ in range(dist.get_world_size(group))]
    dist.all_gather(out, t, group=group)
    return [int(x.item()) for x in out]


def max_over_ranks(value, group=None):
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
