"""Partitioning of the FIR work across GPUs (one process per GPU).

Rows of a batch and ragged signals are independent units, so they are split
across ranks with no exchange on the data path.  The only reduction is the tap
gradient of a data-parallel backward pass (every rank holds a partial dL/dh over
its rows), summed in FP64 with one all-reduce of L values.
"""
from __future__ import annotations

import numpy as np


def row_shard(batch: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous block of rows for `rank`: (first row, row count); sizes differ by at most 1."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("row_shard: need 0 <= rank < world")
    base, extra = divmod(batch, world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def ragged_shard(work: np.ndarray, world: int) -> list[np.ndarray]:
    """Split ragged signals over ranks by greedy longest-first assignment of their work
    (e.g. output samples x taps); returns the signal indices of every rank, each sorted."""
    work = np.asarray(work, dtype=np.float64)
    order = np.argsort(-work, kind="stable")
    load = np.zeros(world)
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += work[i]
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def reduce_tap_grad(dh, group=None):
    """Sum a per-rank tap gradient over all ranks in FP64 (torch tensor, in place)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return dh
    acc = dh.to(torch.float64)
    dist.all_reduce(acc, op=dist.ReduceOp.SUM, group=group)
    dh.copy_(acc.to(dh.dtype))
    return dh
