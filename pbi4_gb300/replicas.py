"""Runs on N GPUs of one node: independent replicas, one process per GPU.

The estimator path does not shard.  Every rank measures whole boxes on its own
GPU (weak scaling: per-GPU work is fixed as N grows) and no data-path
collective exists.  The only cross-rank steps are on the host: a barrier
around a timed region, the maximum over ranks of its elapsed time, and, for a
job over many boxes (a set of mocks or realisations, which the reference runs
one process per catalogue), the split of the box list across ranks and the
gather of the per-box results on rank 0.

The process group is NCCL on GPU runs (launched by torchrun) and gloo in the
CPU tests; the functions here are the same for both.
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def env():
    """(world, rank, local_rank) from the torchrun environment (1, 0, 0 when absent)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None):
    """Join the process group when WORLD_SIZE > 1 and return (world, rank, local_rank).

    backend defaults to "nccl" when CUDA is available, else "gloo".  On CUDA the
    process is bound to its LOCAL_RANK device first, when that device exists (a
    gloo group of more ranks than GPUs, as in the CPU tests, binds none)."""
    world, rank, local = env()
    dev = local if world > 1 else 0
    if torch.cuda.is_available() and dev < torch.cuda.device_count():
        torch.cuda.set_device(dev)
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return world, rank, local


def _active():
    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def barrier():
    if _active():
        dist.barrier()


def _device():
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def max_over_ranks(x: float) -> float:
    """Largest x over all ranks (x itself on a single process)."""
    if not _active():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float) -> float:
    if not _active():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard(n_boxes: int, world: int, rank: int) -> list[int]:
    """Box indices of `rank`: round-robin, so ranks differ by at most one box."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    return list(range(rank, n_boxes, world))


def throughput(boxes_all_ranks: int, seconds_max: float) -> float:
    """Whole-job boxes/s: the boxes all ranks processed over the slowest rank's time."""
    if seconds_max <= 0:
        raise ValueError("elapsed time must be positive")
    return boxes_all_ranks / seconds_max


def gather_results(local: dict[int, object]):
    """Merge {box index: result} dictionaries of all ranks on rank 0 (None elsewhere)."""
    if not _active():
        return dict(local)
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(local, out, dst=0)
    if dist.get_rank() != 0:
        return None
    merged = {}
    for part in out:
        dup = merged.keys() & part.keys()
        if dup:
            raise RuntimeError(f"boxes {sorted(dup)} measured on more than one rank")
        merged.update(part)
    return merged


def run_boxes(n_boxes: int, measure, world: int | None = None, rank: int | None = None):
    """Measure boxes 0..n_boxes-1 across the ranks: this rank runs its shard through
    measure(i) and rank 0 returns {i: result} for all boxes (None on other ranks)."""
    if world is None or rank is None:
        world, rank = (dist.get_world_size(), dist.get_rank()) if _active() else (1, 0)
    mine = {i: measure(i) for i in shard(n_boxes, world, rank)}
    res = gather_results(mine)
    if res is not None and sorted(res) != list(range(n_boxes)):
        raise RuntimeError(f"gathered boxes {sorted(res)} != 0..{n_boxes - 1}")
    return res
