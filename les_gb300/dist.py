"""Replica aggregation for multi-GPU runs.

Members are independent, so N GPUs run N replicas with no data-path
collective; the only cross-rank operation is the timing reduction of the
benchmark: the slowest rank's time and the sum of all ranks' grid-point steps.
"""
import os


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def aggregate(local_ms, local_pt_steps, device=None):
    """Return (max-over-ranks ms, total pt-steps, whole-job pt-steps/s)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_ms, local_pt_steps, local_pt_steps / (local_ms / 1e3)
    t = torch.tensor([local_ms], dtype=torch.float64, device=device)
    p = torch.tensor([float(local_pt_steps)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    ms, pts = float(t.item()), float(p.item())
    return ms, pts, pts / (ms / 1e3)
