"""Multi-process band detection: contiguous pattern shards per rank, no collective in the path.

Patterns are independent, so each rank (one process per GPU, launched by torchrun) takes a
contiguous slice of the batch, runs ``find_bands`` on its own device, and keeps its records.
The only communication is optional and host-side: ``gather_records`` concatenates the
per-rank record arrays on rank 0 (torch.distributed object gather), and ``max_time`` reduces
a timing to its maximum over ranks.  The reference distributes the same way at the
application level (Ray GPU workers over pattern chunks, _ebsd_index_parallel.py:505-760).
"""
from __future__ import annotations

import numpy as np

__all__ = ["shard_bounds", "find_bands_sharded", "find_bands_file_sharded", "gather_records", "max_time"]


def shard_bounds(n, rank, world):
    """[start, stop) of rank's contiguous share of n items (sizes differ by at most one)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(n), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def find_bands_sharded(bd, patterns, rank, world, **kwargs):
    """This rank's records: ``bd.find_bands`` on its shard of ``patterns``.
    Returns (start, records)."""
    s, e = shard_bounds(len(patterns), rank, world)
    return s, bd.find_bands(patterns[s:e], **kwargs)


def find_bands_file_sharded(bd, path, rank, world, **kwargs):
    """This rank's records from a pattern file (UP1 / UP2, .ebsp, .pat): its contiguous share
    of the file's patterns, streamed by ``bd.find_bands_file`` -- each rank reads only its own
    byte ranges.  Returns (start, records)."""
    from .ebsd_pattern import get_pattern_file_obj
    n = int(get_pattern_file_obj(path).nPatterns)
    s, e = shard_bounds(n, rank, world)
    if e == s:
        return s, np.zeros((0, bd.nBands), dtype=bd.dataType)
    return s, bd.find_bands_file(path, patStart=s, nPat=e - s, **kwargs)


def gather_records(start, records, group=None):
    """Rank 0 receives all shards in pattern order (others get None)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world if dist.get_rank(group) == 0 else None
    dist.gather_object((start, records), parts, dst=0, group=group)
    if parts is None:
        return None
    parts.sort(key=lambda p: p[0])
    return np.concatenate([p[1] for p in parts])


def max_time(seconds, group=None):
    """Maximum of a per-rank duration over all ranks."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
