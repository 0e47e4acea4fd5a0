"""Multi-GPU runs of the hot path as independent replicas.

Row windows are independent, so the path needs no exchange between GPUs:
with N ranks (one process per GPU, launched by torchrun) every rank runs its
own whole copy of the workload.  The job's step time is the slowest rank's,
and its throughput counts the units of every rank (weak scaling).  These
helpers hold that host-side logic; they work on any torch.distributed
backend (nccl on GPUs, gloo on CPU).
"""
import os


def env_rank():
    """(rank, local_rank, world_size) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks (the values
    unchanged in a single-process run)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def aggregate_rate(units_per_replica, ms_per_step, world):
    """Units per second of the whole job: every rank processed its own
    `units_per_replica` in (at most) `ms_per_step`."""
    return world * units_per_replica / (ms_per_step * 1e-3)


def reports(rank):
    """Only rank 0 prints the job's line."""
    return rank == 0
