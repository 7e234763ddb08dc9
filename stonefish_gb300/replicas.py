"""Multi-GPU use of the wrench step: replicas only.

Bodies are independent and the ocean is read-only, so there is no exchange
between GPUs on the data path.  Each rank evaluates its own bodies (a
contiguous slice of the batch, or a full replica of a benchmark workload);
the only collective is the timing reduction of the benchmark: the elapsed
time is the maximum over ranks and the whole-job rate counts the units of
all ranks.
"""
from __future__ import annotations


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) slice of n bodies for this rank (sizes differ by
    at most one, every body in exactly one slice)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_over_ranks(x: float, dist=None, device: str = "cpu") -> float:
    """Maximum of x over the ranks of the default process group (x itself
    when dist is None)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units per second of the whole job: every rank processed
    units_per_rank in the (max-over-ranks) time."""
    return world * units_per_rank / seconds
