"""Replica sharding across GPUs (one process per GPU, no data-path collective).

Independent systems (ensemble replicas, served jobs) are split across ranks
by a greedy longest-processing-time bin packing of their work (particles x
steps); each rank advances its share in its own engine, and only the timing
and the work totals are combined: the slowest rank's time and the sum of the
work.  A single system is not split (the reference has no domain
decomposition).
"""
import os


def rank_env():
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def partition(weights, nparts):
    """Indices of `weights` for each of `nparts` ranks: heaviest item first to
    the least-loaded rank (ties: lower rank, then lower index).  Deterministic,
    so every rank computes the same split without communicating; each part's
    indices come back in ascending order."""
    if nparts < 1:
        raise ValueError("nparts must be positive")
    order = sorted(range(len(weights)), key=lambda k: (-weights[k], k))
    load = [0.0] * nparts
    parts = [[] for _ in range(nparts)]
    for k in order:
        r = min(range(nparts), key=lambda q: (load[q], q))
        parts[r].append(k)
        load[r] += weights[k]
    return [sorted(p) for p in parts]


def combine(work, ms, device=None):
    """(sum of work over ranks, max of ms over ranks); the identity without a
    process group.  `device` is where the reduction tensors live (a CUDA
    device for NCCL, the CPU for gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(work), float(ms)
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(w.item()), float(t.item())
