"""Replica runs: one process per GPU, each stepping its own independent
simulation (seeded by rank), timed with a barrier on both sides and reduced
with the maximum over ranks.  The path has no exchange step: the workloads
shard by instance, so there is no collective on the data path; the only
collectives are the barrier and the max of the timings.
"""
from __future__ import annotations

import os

import torch


def dist_env():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend=None):
    world, rank, _ = dist_env()
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"),
                                    rank=rank, world_size=world)
    return world, rank


def _device():
    import torch.distributed as dist
    return torch.device("cuda", torch.cuda.current_device()) \
        if dist.get_backend() == "nccl" else torch.device("cpu")


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def max_over_ranks(x: float) -> float:
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def throughput(cells_per_rank: int, steps: int, ms_total_max: float, world: int) -> float:
    """Whole-job Mcell-steps/s: every rank's cells over the slowest rank's time."""
    return world * cells_per_rank * steps / (ms_total_max * 1e-3) / 1e6


def finalize():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
