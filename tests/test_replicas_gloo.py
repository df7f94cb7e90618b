"""Source sharding over replicas, exercised on CPU with the gloo backend and
world size 2 (the GPU path shards the same way, one process per GPU, with no
collective while traversing). Each rank computes its shard's rows with the
oracle, the rows are all-gathered, and the result must equal the
single-process answer byte for byte."""
import os
import socket

import numpy as np
import pytest

from webgpu_bfs_gb300.replicas import shard_bounds, shard_sources


def test_shard_bounds_cover_disjoint_balanced():
    for S in (0, 1, 2, 3, 7, 512, 513, 2047):
        for world in (1, 2, 3, 4, 8):
            spans = [shard_bounds(S, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == S
            for (b0, e0), (b1, e1) in zip(spans, spans[1:]):
                assert e0 == b1
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(5, 2, 2)
    assert list(shard_sources([9, 8, 7, 6, 5], 1, 2)) == [6, 5]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import webgpu_bfs_gb300 as m
        from oracle import oracle
        from webgpu_bfs_gb300.replicas import run_sharded
        g = m.wilson_grid(30, 20, 15, 3)
        src = m.sample_sources(g, 37, 5)
        V = g.num_vertices
        rows = run_sharded(lambda s: oracle.ms_bfs_fifo(V, g.row_offsets, g.col_indices, s),
                           src, V, rank, world)
        q.put((rank, rows.tobytes()))
    finally:
        dist.destroy_process_group()


def test_gloo_world2_sharded_rows_equal_single_process(oracle):
    import torch.multiprocessing as mp
    import webgpu_bfs_gb300 as m
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    g = m.wilson_grid(30, 20, 15, 3)
    src = m.sample_sources(g, 37, 5)
    want = oracle.ms_bfs_fifo(g.num_vertices, g.row_offsets, g.col_indices, src)
    assert got[0] == got[1] == want.tobytes()
