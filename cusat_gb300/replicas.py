"""Multi-GPU runs of the FEC path: independent replicas, no data exchange.

Frames are independent units (each is demapped, decoded and checked alone),
so N ranks either decode disjoint shards of one frame list or run N
replicas of a workload; the only collectives are the timing and counting
reductions of a benchmark (max of the ranks' times, sum of their frames).
They run over whatever process group is initialised (NCCL on GPUs, gloo on
CPUs in the tests).
"""


def shard(n_items, rank, world):
    """Contiguous [start, stop) of n_items for `rank`: sizes differ by <= 1."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank outside the world")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def reduce_timing(values, device=None):
    """All-reduce MAX of per-rank times (a list of floats); identity when no
    process group is initialised."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def reduce_sum(values, device=None):
    """All-reduce SUM of per-rank counts (frames, bits, errors)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.cpu()]
