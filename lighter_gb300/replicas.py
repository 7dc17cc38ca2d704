"""Multi-GPU runs of the bake are replicas: each rank bakes its own copy of the
workload on its own GPU, with no data-path collective (a bake has no exchange
step). The ranks meet only to time the run: a barrier on both sides of the
timed region and one reduction of the results (sum of the work, max of the
times), over gloo so that it runs without GPUs as well."""
from __future__ import annotations

import os


def init():
    """(world, rank, local_rank, dist or None) from the torchrun environment."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if not dist.is_initialized():
            dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def aggregate(dist, work: float, *times: float):
    """Whole-job work (sum over ranks) and the slowest rank's times (max)."""
    if dist is None:
        return (float(work), *[float(t) for t in times])
    import torch
    w = torch.tensor([float(work)], dtype=torch.float64)
    t = torch.tensor([float(x) for x in times], dtype=torch.float64)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return (w.item(), *t.tolist())
