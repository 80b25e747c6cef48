"""Independent replicas across GPUs.

The WCSPH step of one scene has no data exchange to distribute (a single scene
would need an x-slab halo exchange, not built), so N GPUs run N independent
scenes.  Ranks meet only to time the run: a barrier before and after, the
slowest rank's time, and the particle updates summed over ranks."""


def aggregate(dist, seconds, units, device="cpu"):
    """Return (max seconds over ranks, summed units over ranks).  `dist` is
    torch.distributed (or None for a single process)."""
    if dist is None or not dist.is_initialized():
        return float(seconds), float(units)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def replica_seed(base_seed, rank):
    """Each replica advances its own seeded scene."""
    return int(base_seed) + 7919 * int(rank)
