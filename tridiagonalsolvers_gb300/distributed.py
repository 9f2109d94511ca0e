"""Multi-GPU host logic.  Systems are independent, so a batch shards by system
with no exchange on the data path: rank r solves its own contiguous slice of
systems.  The only collectives are for timing (barrier, max over ranks) and an
optional gather of results for checking; there is no collective inside a solve.
"""
from __future__ import annotations


def shard_range(num_systems: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of the systems owned by `rank`: contiguous, sizes differing
    by at most one, covering every system exactly once."""
    if world <= 0 or not 0 <= rank < world or num_systems < 0:
        raise ValueError("bad rank/world/num_systems")
    q, r = divmod(num_systems, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over the default process group (identity when not
    initialised)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
