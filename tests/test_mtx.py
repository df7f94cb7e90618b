"""Matrix Market reader (CPU): msbfs_mtx_parse / msbfs_mtx_read against the
oracle's line-by-line restatement of MtxReader::parse (crates/core/src/mtx.rs)
and against the behaviours the reference's own tests assert (mtx.rs:277-428:
header variants, symmetric expansion with comments, self-loop removal and
deduplication, zero index, out-of-bounds index, a path-shaped road mock)."""
import numpy as np
import pytest

BANNER = "%%MatrixMarket matrix coordinate pattern "


def _same_as_oracle(native, oracle, text):
    try:
        want = oracle.mtx_parse(text)
    except oracle.MtxOracleError as e:
        with pytest.raises(native.MtxError) as got:
            native.parse_mtx(text)
        assert got.value.kind == e.kind, text
        assert got.value.line_number == e.line, text
        assert str(got.value) == str(e), text
        return None
    g = native.parse_mtx(text)
    V, ro, ci = want
    assert g.num_vertices == V
    assert np.array_equal(g.row_offsets, ro) and np.array_equal(g.col_indices, ci)
    return g


def test_header_variants(native, oracle):
    ok = ["%%MatrixMarket matrix coordinate pattern symmetric",
          "%%matrixmarket MATRIX COORDINATE real general",
          "%%MatrixMarket matrix coordinate integer skew-symmetric",
          "%%MatrixMarket matrix coordinate complex hermitian",
          "\n\n  %%MatrixMarket   matrix coordinate pattern general  "]
    for h in ok:
        g = _same_as_oracle(native, oracle, h + "\n3 3 1\n1 2\n")
        assert g is not None and g.num_vertices == 3
    bad = {"%%MatrixMarket matrix array real general": "UnsupportedFormat",
           "%%MatrixMarket matrix coordinate real": "InvalidHeader",
           "%MatrixMarket matrix coordinate real general": "InvalidHeader",
           "%%MatrixMarket vector coordinate real general": "InvalidHeader",
           "%%MatrixMarket matrix sparse real general": "InvalidHeader",
           "%%MatrixMarket matrix coordinate double general": "InvalidHeader",
           "%%MatrixMarket matrix coordinate real upper": "InvalidHeader",
           "% a comment first\n%%MatrixMarket matrix coordinate real general": "InvalidHeader"}
    for h, kind in bad.items():
        with pytest.raises(native.MtxError) as e:
            native.parse_mtx(h + "\n3 3 1\n1 2\n")
        assert e.value.kind == kind
        _same_as_oracle(native, oracle, h + "\n3 3 1\n1 2\n")
    for text in ("", "\n  \n"):
        with pytest.raises(native.MtxError) as e:
            native.parse_mtx(text)
        assert e.value.kind == "InvalidHeader"
        _same_as_oracle(native, oracle, text)


def test_symmetric_pattern_with_comments(native, oracle):
    text = (BANNER + "symmetric\n% first comment\n%second\n5 5 4\n1 2\n2 3\n% inner\n"
            "3 4\n\n4 5\n")
    g = _same_as_oracle(native, oracle, text)
    assert g.num_edges == 8
    assert list(g.col_indices[g.row_offsets[1]:g.row_offsets[2]]) == [0, 2]
    assert native.GpuBfsEngine.select_auto_method  # the graph is an ordinary CsrGraph
    assert oracle.is_symmetric(g.num_vertices, g.row_offsets, g.col_indices)


def test_self_loops_and_duplicates(native, oracle):
    text = ("%%MatrixMarket matrix coordinate real general\n4 4 7\n1 1 1.0\n1 3 2.5\n"
            "1 3 -3.0\n2 4 1e3\n4 4 0.5\n3 1 7\n2 4 8\n")
    g = _same_as_oracle(native, oracle, text)
    assert g.num_edges == 3  # (1,3), (2,4), (3,1); self-loops gone, duplicates merged
    assert list(g.row_offsets) == [0, 1, 2, 3, 3]


def test_zero_and_out_of_range_indices(native, oracle):
    z = BANNER + "general\n% c\n3 3 2\n1 2\n\n0 3\n"
    with pytest.raises(native.MtxError) as e:
        native.parse_mtx(z)
    assert (e.value.kind, e.value.line_number, e.value.row, e.value.col) == ("ZeroIndex", 6, 0, 3)
    o = BANNER + "general\n3 2 1\n3 3\n"
    with pytest.raises(native.MtxError) as e:
        native.parse_mtx(o)
    v = e.value
    assert (v.kind, v.line_number, v.row, v.col, v.max_rows, v.max_cols) == \
        ("IndexOutOfBounds", 3, 3, 3, 3, 2)
    for t in (z, o):
        _same_as_oracle(native, oracle, t)


def test_rectangular_and_dimension_errors(native, oracle):
    g = _same_as_oracle(native, oracle, BANNER + "general\n2 6 2\n1 6\n2 5\n")
    assert g.num_vertices == 6  # max(rows, cols)
    for text in (BANNER + "symmetric\n2 3 1\n1 2\n",       # symmetric must be square
                 BANNER + "general\n3 3\n1 2\n",           # two tokens
                 BANNER + "general\n3 x 1\n1 2\n",         # invalid digit
                 BANNER + "general\n3 -3 1\n",             # sign
                 BANNER + "general\n99999999999999999999 3 1\n",  # overflow
                 BANNER + "general\n% only comments\n\n"):  # no dimension line
        with pytest.raises(native.MtxError) as e:
            native.parse_mtx(text)
        assert e.value.kind == "InvalidDimensions"
        _same_as_oracle(native, oracle, text)


def test_coordinate_line_errors(native, oracle):
    for bad in ("2", "1 x", "1.0 2", "-1 2"):
        text = BANNER + "general\n3 3 2\n1 2\n" + bad + "\n"
        with pytest.raises(native.MtxError) as e:
            native.parse_mtx(text)
        assert (e.value.kind, e.value.line_number) == ("InvalidCoordinateLine", 4)
        _same_as_oracle(native, oracle, text)
    g = _same_as_oracle(native, oracle, BANNER + "general\n3 3 1\n+1 +3\n")
    assert g.num_edges == 1


def test_road_mock_path(native, oracle):
    """A path-shaped road mock: degrees 1, 2, ..., 2, 1."""
    n = 9
    text = BANNER + f"symmetric\n% road mock\n{n} {n} {n - 1}\n" + "".join(
        f"{i} {i + 1}\n" for i in range(1, n))
    g = _same_as_oracle(native, oracle, text)
    deg = np.diff(g.row_offsets)
    assert g.num_edges == 2 * (n - 1) and deg.max() == 2 and deg[0] == 1 and deg[-1] == 1
    d = oracle.ms_bfs_fifo(g.num_vertices, g.row_offsets, g.col_indices, [0])
    assert list(d) == list(range(n))


def _big_text(rng, n_rows, n_entries, crlf=False, bad_at=None):
    eol = "\r\n" if crlf else "\n"
    r = rng.integers(1, n_rows + 1, n_entries)
    c = rng.integers(1, n_rows + 1, n_entries)
    out = [BANNER + "symmetric", "% generated", f"{n_rows} {n_rows} {n_entries}"]
    for k in range(n_entries):
        if k % 977 == 0:
            out.append("% a comment between entries")
        if k % 1313 == 0:
            out.append("")
        out.append(f"{r[k]} {c[k]}" if bad_at != k else f"{r[k]} 0")
    return eol.join(out) + eol


@pytest.mark.parametrize("crlf", [False, True])
def test_large_file_parallel_chunks(native, oracle, crlf):
    """Several MB of entries are parsed in parallel chunks; the graph and the
    line number of an error deep in the file match the line-by-line oracle."""
    rng = np.random.default_rng(7 + crlf)
    text = _big_text(rng, 50000, 400000, crlf)
    assert len(text) > 4 << 20
    _same_as_oracle(native, oracle, text)
    bad = _big_text(rng, 50000, 400000, crlf, bad_at=312345)
    with pytest.raises(native.MtxError) as e:
        native.parse_mtx(bad)
    assert e.value.kind == "ZeroIndex"
    _same_as_oracle(native, oracle, bad)


def test_read_file(native, tmp_path):
    p = tmp_path / "g.mtx"
    p.write_text(BANNER + "symmetric\n3 3 2\n1 2\n2 3\n")
    g = native.read_mtx(p)
    assert g.num_vertices == 3 and g.num_edges == 4
    with pytest.raises(native.MtxError) as e:
        native.read_mtx(tmp_path / "missing.mtx")
    assert e.value.kind == "Io"


@pytest.mark.parametrize("threads", ["1", "3", None])
def test_host_thread_counts_give_the_generated_graph(native, monkeypatch, threads):
    """A generated R-MAT graph written as a symmetric pattern file (its lower
    triangle) parses back to the same CSR whatever the number of host threads
    (MSBFS_HOST_THREADS): the entries are split into per-thread chunks and the
    CSR is built from source-vertex partitions, both sized by the count."""
    import bench
    if threads:
        monkeypatch.setenv("MSBFS_HOST_THREADS", threads)
    else:
        monkeypatch.delenv("MSBFS_HOST_THREADS", raising=False)
    g = native.generate_graph500_rmat(15, 16, 5)
    text, entries = bench.mtx_text(g)
    assert entries * 2 == g.num_edges and len(text) > 3 << 20  # several 1 MB chunks
    p = native.parse_mtx(text)
    assert p.num_vertices == g.num_vertices
    assert np.array_equal(p.row_offsets, g.row_offsets)
    assert np.array_equal(p.col_indices, g.col_indices)
