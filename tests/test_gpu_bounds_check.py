"""The bounds-checked build of the engine (-DMSBFS_BOUNDS_CHECK), on the GPU.

That build range-checks the level kernels' indices (in-neighbour ids, work
list entries, hub slices, queue entries and capacity, out-edge targets) and
bounds their claim loops; a failed check records its site and the call
returns MSBFS_ERR_CUDA ("bounds check failed at site N") instead of
faulting. It stands in for a memory checker, which this GPU pool does not
offer. Here it is built beside the default library and runs representative
traversals in a child process (the library is loaded once per process):
every result must equal the oracle's and no check may fire.
"""
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = textwrap.dedent("""
    import sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    import webgpu_bfs_gb300 as m
    from oracle import oracle
    cases = [
        (m.generate_graph500_rmat(14, 16, 3), 700, "PushPullAdaptive"),
        (m.generate_graph500_rmat(14, 16, 3), 512, "MultiWordBitParallel"),
        (m.generate_rmat(12, 8, 0.57, 0.19, 0.19, 0.05, 4, directed=True), 300, "Auto"),
        (m.wilson_grid(120, 100, 200, 5), 256, "PushPullAdaptive"),  # > 256 levels
        (m.path_graph(1500), 4, "BitParallel64"),
        (m.generate_erdos_renyi_np(5000, 8 / 4999, 2), 2048, "PushPullAdaptive"),
    ]
    eng = m.GpuBfsEngine(m.GpuBfsMethod.Auto)
    eng.set_tuning(max_words_per_pass=64)  # W = 64 passes too
    for g, S, meth in cases:
        src = np.random.default_rng(S).integers(0, g.num_vertices, S).astype(np.uint32)
        got = eng.run_ms_bfs_with_method(m.GpuBfsMethod[meth], g, src)
        want = oracle.ms_bfs_threaded(g.num_vertices, g.row_offsets, g.col_indices, src)
        assert np.array_equal(got, want), (g.num_vertices, S, meth)
        print("ok", g.num_vertices, S, meth, eng.last_stats["levels"], flush=True)
    eng.close()
""")


def test_bounds_checked_build_matches_oracle(tmp_path):
    from webgpu_bfs_gb300 import build as b
    lib = b.build_native(defines=["MSBFS_BOUNDS_CHECK"], out_dir=tmp_path / "check")
    env = dict(os.environ, MSBFS_LIB=str(lib))
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert r.stdout.count("ok ") == 6
