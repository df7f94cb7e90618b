"""The Python mirror's structs match include/msbfs.h byte for byte (CPU).

A small C program compiled against the header prints sizeof and the
offsetof of every field; the ctypes definitions in webgpu_bfs_gb300/_native.py
(and the numpy view of msbfs_source_stats) must agree, so a field added to
or renamed in the header without its mirror fails here instead of silently
shifting the fields after it.
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

# C struct name -> (ctypes mirror name, [(C field, mirror field)])
STRUCTS = {
    "msbfs_stats": ("Stats", [
        ("method", "method"), ("path", "path"), ("passes", "passes"),
        ("words_per_vertex", "words_per_vertex"), ("levels", "levels"),
        ("push_levels", "push_levels"), ("pull_levels", "pull_levels"),
        ("cta_cluster", "cta_cluster"), ("reached_pairs", "reached_pairs"),
        ("gpu_ms", "gpu_ms")]),
    "msbfs_level_record": ("LevelRecord", [
        ("pass", "pass_"), ("level", "level"), ("dir", "dir"),
        ("frontier_vertices", "frontier_vertices"), ("frontier_entries", "frontier_entries"),
        ("active", "active"), ("edges", "edges"), ("new_vertices", "new_vertices"),
        ("new_pairs", "new_pairs"), ("rows", "rows"), ("device_ms", "device_ms"),
        ("event_ms", "event_ms")]),
    "msbfs_csr": ("Csr", [
        ("num_vertices", "num_vertices"), ("num_edges", "num_edges"),
        ("row_offsets", "row_offsets"), ("col_indices", "col_indices")]),
    "msbfs_server_config": ("ServerConfig", [
        ("slots", "slots"), ("max_sources_per_launch", "max_sources_per_launch"),
        ("hbm_budget_bytes", "hbm_budget_bytes"), ("method", "method"),
        ("express_slots", "express_slots"), ("small_sources", "small_sources"),
        ("general_sm_percent", "general_sm_percent"), ("reserved", "reserved")]),
    "msbfs_request_info": ("RequestInfo", [
        ("latency_ms", "latency_ms"), ("queue_ms", "queue_ms"),
        ("launches", "launches"), ("status", "status")]),
    "msbfs_mtx_error": ("MtxErrorInfo", [
        ("kind", "kind"), ("line_number", "line_number"), ("row", "row"), ("col", "col"),
        ("max_rows", "max_rows"), ("max_cols", "max_cols"), ("message", "message")]),
    "msbfs_tuning": ("Tuning", [
        ("max_words_per_pass", "max_words_per_pass"), ("alpha", "alpha"), ("beta", "beta"),
        ("hub_split", "hub_split"), ("bitmap_div", "bitmap_div"),
        ("warp_scan_degree", "warp_scan_degree"), ("from_cache", "from_cache"),
        ("trials", "trials"), ("level_path", "level_path"), ("ms", "ms"),
        ("default_ms", "default_ms"), ("class_name", "class_name")]),
    "msbfs_batch_graph": ("BatchGraph", [
        ("num_vertices", "num_vertices"), ("num_edges", "num_edges"),
        ("row_offsets", "row_offsets"), ("col_indices", "col_indices"),
        ("sources", "sources"), ("num_sources", "num_sources")]),
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "msbfs.h"', "int main(void) {"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for cf, _ in fields:
            lines.append(f'  printf("{cname} {cf} %zu\\n", offsetof({cname}, {cf}));')
    for cf in ("distance_sum", "eccentricity", "reached"):
        lines.append(f'  printf("msbfs_source_stats {cf} %zu\\n", offsetof(msbfs_source_stats, {cf}));')
    lines.append('  printf("msbfs_source_stats size %zu\\n", sizeof(msbfs_source_stats));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([cc, "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        s, f, v = line.split()
        table[(s, f)] = int(v)
    return table


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_mirror_matches_header(c_layout, cname):
    from webgpu_bfs_gb300 import _native
    mirror_name, fields = STRUCTS[cname]
    mirror = getattr(_native, mirror_name)
    assert [f for f, _ in mirror._fields_] == [m for _, m in fields], "field list"
    assert C.sizeof(mirror) == c_layout[(cname, "size")]
    for cf, mf in fields:
        assert getattr(mirror, mf).offset == c_layout[(cname, cf)], f"{cname}.{cf}"


def test_source_stats_view_matches_header(c_layout):
    from webgpu_bfs_gb300 import _native
    dt = np.dtype(_native.SOURCE_STATS_DTYPE)
    assert dt.itemsize == c_layout[("msbfs_source_stats", "size")]
    for name in dt.names:
        assert dt.fields[name][1] == c_layout[("msbfs_source_stats", name)]
