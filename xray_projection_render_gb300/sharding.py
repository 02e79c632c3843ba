"""Replicas on several GPUs: the reference shards its work by view index
(``--jobs_modulo``, main.go:244), and so does this engine -- view (or scene)
k goes to rank k mod N, with no exchange between ranks.  The only
cross-rank step is the job's timing: the slowest rank's time and the sum of
the units all ranks processed."""
from __future__ import annotations


def shard(items, rank: int, world: int):
    """The items of `rank` (k mod world == rank), in order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    return list(items)[rank::world]


def job_time(t_local: float, units_local: float, device=None):
    """(max time over ranks, total units over ranks) through
    torch.distributed (any backend); the local values when it is not
    initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(t_local), float(units_local)
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
