"""Replica orchestration for multi-GPU runs.

One instance of the hot path (one grid) runs on one GPU; there is no
data-path exchange between GPUs.  With N processes (one per GPU, launched by
torchrun) every rank solves its own instance; the ranks only meet at a
barrier before and after a timed region and agree on the slowest rank's
time.  The process group is gloo or nccl depending on the device.
"""

import os

import torch
import torch.distributed as dist


def init_from_env(backend=None):
    """Initialise the process group from RANK/WORLD_SIZE/MASTER_* if present.
    Returns (rank, world_size, local_rank)."""
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault('MASTER_ADDR', '127.0.0.1')
        if backend is None:
            backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        dist.init_process_group(backend=backend, rank=rank, world_size=world)
    return rank, world, local


def barrier():
    if dist.is_initialized():
        if dist.get_backend() == 'nccl':
            dist.barrier(device_ids=[torch.cuda.current_device()])
        else:
            dist.barrier()


def max_over_ranks(value):
    """Maximum of a float over all ranks (the job's time is the slowest rank's)."""
    if not dist.is_initialized():
        return float(value)
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value):
    if not dist.is_initialized():
        return float(value)
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def finalize():
    if dist.is_initialized():
        dist.destroy_process_group()
