"""Data-parallel replicas of the transport path (one process per GPU).

Primaries are independent, so ranks share no data: rank r of W transports,
at step s, the primaries of block s*W + r, whose random streams are those
of the global primary indices (s*W + r)*n .. (s*W + r)*n + n - 1.  Together
the ranks cover consecutive blocks with disjoint streams, and the job's
result is the same as one process transporting every block.  The only
collective is the reduction of the timing and the counts at the end.
"""
from __future__ import annotations


def block_index(step: int, rank: int, world: int) -> int:
    """Primary block a rank transports at a step."""
    return step * world + rank


def first_primary(step: int, rank: int, world: int, n: int) -> int:
    """Global index of the first primary of the rank's block (stream offset)."""
    return block_index(step, rank, world) * n


def reduce_job(t_local: float, units_local: float, dist=None, device="cpu"):
    """Whole-job figures: the slowest rank's time and the sum of the units
    (particle-steps, rows, ...) over ranks."""
    if dist is None:
        return float(t_local), float(units_local)
    import torch
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
