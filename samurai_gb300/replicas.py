"""Multi-GPU use of the path: independent replicas, no data-path collective.

One large MR mesh does not shard with a single exchange step, so N GPUs run N
independent problems (or N shards of a batch of independent problems), one
process per GPU.  Only the timing and the counts are combined, once, after the
timed region: the slowest rank's time and the sum of the cell-updates.
"""


def reduce_over_ranks(total_ms, cell_updates, world, device="cpu"):
    """(max of total_ms, sum of cell_updates) over the ranks of the default
    process group; the identity when world == 1."""
    if world == 1:
        return float(total_ms), float(cell_updates)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    n = torch.tensor([float(cell_updates)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), float(n.item())


def shard_instances(sizes, rank, world):
    """Indices of the independent instances rank `rank` of `world` advances:
    greedy balance of the given per-instance sizes (largest first onto the
    least-loaded rank), deterministic on every rank."""
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0.0] * world
    owner = [0] * len(sizes)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += sizes[i]
    return [i for i in range(len(sizes)) if owner[i] == rank]
