"""Replica runs under torchrun: one process per GPU, each training its own
field on its own copy of the workload (the path's units, the leaves of a
field, need no exchange between replicas).  Ranks meet only around the timed
region: a barrier before and after, and the maximum of each rank's timings.

The process group is plumbing: NCCL on GPUs, gloo for the CPU tests.
"""

import datetime

import torch
import torch.distributed as dist


def init(backend="nccl", timeout_s=120.0):
    """Joins the process group described by the torchrun environment
    (RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT)."""
    dist.init_process_group(backend, timeout=datetime.timedelta(seconds=timeout_s))


def active():
    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def barrier(device=None):
    """All ranks arrive; then (on a GPU) all of this rank's queued work is done."""
    if active():
        dist.barrier()
    if device is not None and torch.device(device).type == "cuda":
        torch.cuda.synchronize()


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of each rank's float values (the slowest replica
    sets the job's time)."""
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if active():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job_ms_per_unit(ms_per_step, samples_per_step, unit_samples, world):
    """Time of the whole job per `unit_samples` samples when `world` replicas
    each process `samples_per_step` samples in `ms_per_step` (weak scaling:
    per-replica work is fixed, the job processes world times as many)."""
    return ms_per_step * unit_samples / (samples_per_step * world)


def shutdown():
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
