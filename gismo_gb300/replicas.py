"""Replicas across GPUs: one process per GPU (torchrun), each assembling and solving its own
independent problem, with no exchange on the data path. The only cross-rank communication is
the timing reduction of the benchmark: the slowest rank's time and the units all ranks processed,
so that whole-job throughput = sum of units / max time (weak scaling)."""
from __future__ import annotations


def replica_seed(seed: int, rank: int) -> int:
    """Seed of rank `rank`'s independent problem (rank 0 keeps the base seed)."""
    return seed + 1000 * rank


def reduce_max_sum(dist, t_ms: float, units: float, device="cpu"):
    """(max of t_ms over ranks, sum of units over ranks); the local pair without a process group.
    `dist` is torch.distributed after init_process_group (nccl with device "cuda", gloo with "cpu")."""
    if dist is None:
        return float(t_ms), float(units)
    import torch
    t = torch.tensor([float(t_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
