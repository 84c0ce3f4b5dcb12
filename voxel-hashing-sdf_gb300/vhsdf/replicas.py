"""Multi-GPU by replicas: independent frame streams or scenes per rank.

A volume never spans GPUs; ranks share nothing on the data path.  The only
collectives reduce the per-rank timings (max) and gather per-rank counts at
the end of a run.  Works with any torch.distributed backend (NCCL on GPUs,
gloo on CPU for tests).
"""


def stream_seed(base_seed, rank):
    """Seed of the synthetic stream a rank fuses (rank 0 keeps the base)."""
    return int(base_seed) + int(rank)


def assign(num_items, rank, world):
    """Round-robin share of `num_items` independent scenes for `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(range(rank, num_items, world))


def reduce_max(values, device=None):
    """Element-wise max over ranks of a list of floats (no-op without a group)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def gather_counts(counts, device=None):
    """All ranks' integer counts, as a list per rank."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(counts), dtype=torch.int64, device=device)
    if not (dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1):
        return [t.tolist()]
    out = [torch.empty_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(out, t)
    return [o.tolist() for o in out]
