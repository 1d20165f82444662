"""Independent replicas across ranks (one process per GPU, no data-path
collective): the only multi-GPU form of this path.  A PT run has no exchange
between GPUs on this path; independent systems or seeds shard with no
communication, and the job's rate is the summed work over the slowest rank's
time.
"""
from __future__ import annotations


def shard(n_items: int, rank: int, world: int) -> slice:
    """Contiguous, balanced share of ``n_items`` for ``rank`` of ``world``
    (the first ``n_items % world`` ranks take one more item)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f'rank {rank} outside a world of {world}')
    base, extra = divmod(int(n_items), int(world))
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def job_rate(units_local: float, seconds_local: float, device=None):
    """(units summed over ranks, seconds of the slowest rank, units/s) with
    two all-reduces on the default process group; the local values when
    torch.distributed is not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(units_local), float(seconds_local), float(units_local) / float(seconds_local)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    t = torch.tensor([float(seconds_local)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()), float(t.item()), float(u.item()) / float(t.item())
