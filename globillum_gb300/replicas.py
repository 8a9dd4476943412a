"""Replica aggregation for multi-GPU runs.

Every path is independent, so N GPUs render N replicas of the workload with
no exchange on the data path; the job's throughput is all ranks' paths over
the slowest rank's time (a max-reduce of the time and a sum-reduce of the
work, the only collectives).
"""
from __future__ import annotations


def aggregate(paths_local: float, ms_local: float, dist=None, device=None) -> tuple[float, float]:
    """Returns (total paths, max ms over ranks); single process without `dist`."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(paths_local), float(ms_local)
    import torch
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    p = torch.tensor([float(paths_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(p.item()), float(t.item())


def mpaths_per_s(paths_total: float, ms_max: float) -> float:
    return paths_total / (ms_max / 1e3) / 1e6
