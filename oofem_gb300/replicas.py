"""Independent replicas, one process per GPU (torchrun): the hot path has no
exchange step, so N ranks each solve their own mesh and only the timing is
combined -- the step time of the job is the slowest rank's, the work is the sum
over ranks. Works with NCCL on GPUs and with gloo on CPU (tests)."""
from __future__ import annotations

import os


def env():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _reduce(value: float, op_name: str) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(value: float) -> float:
    return _reduce(value, "MAX")


def sum_over_ranks(value: float) -> float:
    return _reduce(value, "SUM")


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def job_throughput(units_local: float, seconds_local: float) -> float:
    """Units of all ranks divided by the slowest rank's time."""
    return sum_over_ranks(units_local) / max_over_ranks(seconds_local)
