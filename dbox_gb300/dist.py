"""Multi-GPU layout of independent worlds: one process per GPU, no collective on
the data path.  Worlds never interact, so ranks either run their own batch
(weak scaling: seed offset per rank) or split one batch into contiguous ranges
(strong scaling); timing is reduced with a max over ranks."""


def world_range(n_worlds, rank, world_size):
    """Contiguous [start, stop) slice of n_worlds for rank (sizes differ by at most one)."""
    base, extra = divmod(n_worlds, world_size)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def rank_seed(seed, rank):
    """Seed of rank's own batch under weak scaling."""
    return seed + 1000 * rank


def max_over_ranks(value, device="cpu"):
    """Maximum of a float over all ranks of the default process group (the value itself if none)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
