"""Source sharding over replicas (one process per GPU).

Each source's BFS is independent, so the multi-source BFS shards by source
with no exchange step: every rank keeps its own resident copy of the graph
and traverses a contiguous block of the sources (rows ``begin .. end`` of the
source-major distance matrix). Nothing is communicated while traversing;
``gather_rows`` only assembles finished rows for callers that want the whole
matrix in one process (it is not part of a timed step).
"""
from __future__ import annotations

from typing import Callable, Optional

import numpy as np


def shard_bounds(num_sources: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced block of sources owned by ``rank``: the first
    ``num_sources % world`` ranks take one source more than the others."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(num_sources, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def shard_sources(sources, rank: int, world: int) -> np.ndarray:
    src = np.ascontiguousarray(np.asarray(sources, dtype=np.uint32))
    b, e = shard_bounds(src.size, rank, world)
    return src[b:e]


def gather_rows(local_rows: np.ndarray, num_sources: int, num_vertices: int, rank: int,
                world: int, group=None) -> np.ndarray:
    """All-gathers every rank's finished rows (u32, source-major) into the
    full ``num_sources * num_vertices`` matrix on every rank, through
    torch.distributed (gloo on CPU tensors, nccl on device tensors)."""
    import torch
    import torch.distributed as dist

    if world == 1:
        return np.ascontiguousarray(local_rows, dtype=np.uint32)
    width = max(shard_bounds(num_sources, r, world)[1] - shard_bounds(num_sources, r, world)[0]
                for r in range(world)) * num_vertices
    b, e = shard_bounds(num_sources, rank, world)
    mine = torch.zeros(width, dtype=torch.int32)
    rows = np.ascontiguousarray(local_rows, dtype=np.uint32).view(np.int32)
    if rows.size != (e - b) * num_vertices:
        raise ValueError("local rows do not match this rank's shard")
    mine[:rows.size] = torch.from_numpy(rows)
    parts = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine, group=group)
    out = np.empty(num_sources * num_vertices, np.uint32)
    for r, t in enumerate(parts):
        rb, re_ = shard_bounds(num_sources, r, world)
        n = (re_ - rb) * num_vertices
        out[rb * num_vertices:rb * num_vertices + n] = t[:n].numpy().view(np.uint32)
    return out


def run_sharded(compute: Callable[[np.ndarray], np.ndarray], sources, num_vertices: int,
                rank: int, world: int, gather: bool = True,
                group: Optional[object] = None) -> np.ndarray:
    """Runs ``compute`` (e.g. ``GpuBfsEngine.run_ms_bfs`` bound to a graph)
    on this rank's shard; returns the local rows, or all rows when
    ``gather``."""
    src = np.ascontiguousarray(np.asarray(sources, dtype=np.uint32))
    local = compute(shard_sources(src, rank, world))
    if not gather:
        return local
    return gather_rows(local, src.size, num_vertices, rank, world, group)
