"""
Replicas on several GPUs: independent tissues (or batches of cables) per
rank, with no exchange on the data path. The only collective is the
timing reduction: the job's time is the slowest rank's, its work the sum.
"""


def shard(n, world, rank):
    """
    The contiguous range ``[start, stop)`` of ``n`` independent units (for
    example the cables of a batch) that rank ``rank`` of ``world`` owns;
    sizes differ by at most one.
    """
    n, world, rank = int(n), int(world), int(rank)
    if world < 1 or not 0 <= rank < world:
        raise ValueError('rank must be in [0, world)')
    return rank * n // world, (rank + 1) * n // world


def combine(device_ms, wall_s, units, world=1, dist=None, device='cpu'):
    """
    Whole-job figures of a replica run: ``(device_ms, wall_s, units)`` with
    the times the maximum over ranks and the units the sum. ``dist`` is
    ``torch.distributed`` (initialised) or None for one rank; ``device``
    holds the reduction tensor ('cuda' for NCCL, 'cpu' for gloo).
    """
    if dist is None or world <= 1:
        return float(device_ms), float(wall_s), int(units)
    import torch
    t = torch.tensor([float(device_ms), float(wall_s)], dtype=torch.float64,
                     device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([int(units)], dtype=torch.int64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t[0]), float(t[1]), int(u[0])
