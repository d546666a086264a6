"""Host graph substrate (CPU only): generators, CSR builder, file formats."""
import numpy as np
import pytest

import dfqbfs as d


def test_generator_determinism():
    a = d.gen_zipf_geometric(5000, 4.7, 2.1, seed=11)
    b = d.gen_zipf_geometric(5000, 4.7, 2.1, seed=11)
    c = d.gen_zipf_geometric(5000, 4.7, 2.1, seed=12)
    assert np.array_equal(a.offsets, b.offsets) and np.array_equal(a.cols, b.cols)
    assert not (np.array_equal(a.offsets, c.offsets) and np.array_equal(a.cols, c.cols))
    r1, r2 = d.gen_rmat(12, 8, seed=5), d.gen_rmat(12, 8, seed=5)
    assert np.array_equal(r1.offsets, r2.offsets) and np.array_equal(r1.cols, r2.cols)
    g1, o1 = d.gen_grid(64, 0.05, seed=2)
    g2, o2 = d.gen_grid(64, 0.05, seed=2)
    assert np.array_equal(g1.cols, g2.cols) and np.array_equal(o1, o2)


def test_zipf_geometric_shape():
    g = d.gen_zipf_geometric(262144, 4.7, 2.1, seed=1)
    assert g.n == 262144
    # mean out-degree 4.7 -> ~1.23M edges
    assert 1.20e6 < g.e < 1.26e6
    deg = g.degrees()
    # no self-loops, no repeated neighbours
    for u in range(0, g.n, 997):
        row = g.cols[g.offsets[u]:g.offsets[u + 1]]
        assert u not in row
        assert len(np.unique(row)) == len(row)
    # power-law in-degree: Zipf(2.1) puts ~64% of each draw on rank 1, and
    # repeats are redrawn, so nearly every vertex with an out-edge points at
    # the heaviest destination once; in-degrees fall off steeply by rank
    indeg = np.sort(np.bincount(g.cols, minlength=g.n))[::-1]
    assert indeg[0] > 0.6 * np.count_nonzero(deg)
    assert indeg[0] > indeg[1] > indeg[9] > indeg[99] > 0
    assert np.count_nonzero(indeg) < 0.05 * g.n
    assert deg[0] > 0  # the configured source 0 is not degenerate


def test_rmat_symmetric_dedup():
    g = d.gen_rmat(12, 16, seed=3)
    assert g.n == 4096
    for u in range(g.n):
        row = g.cols[g.offsets[u]:g.offsets[u + 1]]
        assert np.all(np.diff(row) > 0)  # sorted, unique
        assert u not in row
    # symmetric: (u,v) present iff (v,u) present
    src = np.repeat(np.arange(g.n), g.degrees())
    fwd = set(zip(src.tolist(), g.cols.tolist()))
    assert all((v, u) in fwd for (u, v) in list(fwd)[:5000])


def test_grid_lcc_and_order():
    g, orig = d.gen_grid(100, 0.0, seed=1)
    assert g.n == 10000 and g.e == 2 * 2 * 100 * 99
    assert np.array_equal(orig, np.arange(10000))
    g2, orig2 = d.gen_grid(100, 0.2, seed=1)
    assert g2.n < 10000 and np.all(np.diff(orig2) > 0)  # row-major compact relabel
    for u in range(g2.n):
        row = g2.cols[g2.offsets[u]:g2.offsets[u + 1]]
        assert np.all(np.diff(row) > 0) and len(row) <= 4


def test_csr_from_edges_flags():
    src = [0, 0, 1, 2, 2, 3, 3]
    dst = [1, 1, 2, 2, 0, 3, 0]
    g = d.from_edges(src, dst, 5)
    assert g.offsets.tolist() == [0, 2, 3, 5, 7, 7]
    assert g.cols.tolist() == [1, 1, 2, 2, 0, 3, 0]  # input order kept
    g2 = d.from_edges(src, dst, 5, d.CSR_DEDUP | d.CSR_NO_SELF_LOOPS)
    assert g2.offsets.tolist() == [0, 1, 2, 3, 4, 4]
    assert g2.cols.tolist() == [1, 2, 0, 0]
    g3 = d.from_edges([0, 1], [1, 2], 3, d.CSR_SYMMETRIZE)
    assert g3.offsets.tolist() == [0, 1, 3, 4]
    with pytest.raises(d.DfqError) as e:
        d.from_edges([0], [7], 3)
    assert e.value.name == "EFORMAT"


@pytest.mark.parametrize("fmt", ["snap", "dat", "bin"])
def test_roundtrip(tmp_path, fmt):
    g = d.gen_rmat(10, 8, seed=9)
    g.source = 17
    p = tmp_path / f"g.{fmt}"
    g.save(p, fmt)
    h = d.load(p)
    assert np.array_equal(g.offsets, h.offsets) and np.array_equal(g.cols, h.cols)
    if fmt != "snap":
        assert h.source == 17


def test_snap_reader_details(tmp_path):
    p = tmp_path / "s.txt"
    p.write_text("# Directed graph\n# Nodes: 4 Edges: 3\n# FromNodeId\tToNodeId\n0\t1\n1 2 99\n\n3\t9\n")
    g = d.load(p)
    assert g.n == 10  # ids above the header's N grow N
    assert g.offsets.tolist()[:5] == [0, 1, 2, 2, 3]
    assert g.cols.tolist() == [1, 2, 9]


def test_dat_reader_general_records(tmp_path):
    # rows not back to back: vertex 0 uses edges [2,4), vertex 1 uses [0,2)
    p = tmp_path / "g.dat"
    p.write_text("3 4 1\n2 2\n0 2\n4 0\n2 1\n0 1\n1 1\n2 1\n")
    g = d.load(p)
    assert g.source == 1 and g.n == 3
    assert g.offsets.tolist() == [0, 2, 4, 4]
    assert g.cols.tolist() == [1, 2, 2, 0]


@pytest.mark.parametrize("text", [
    "3 2 0\n0 1\n1 1\n",              # truncated node records
    "2 2 0\n0 1\n1 1\n0 1\n",         # truncated edge records
    "2 1 0\n0 1\n1 5\n0 1\n",         # length past E
    "2 1 0\n0 1\n1 0\n5 1\n",         # edge target out of range
    "x y z\n",                        # not a header
])
def test_dat_malformed(tmp_path, text):
    p = tmp_path / "bad.dat"
    p.write_text(text)
    with pytest.raises(d.DfqError) as e:
        d.load(p)
    assert e.value.name == "EFORMAT"


def test_missing_file():
    with pytest.raises(d.DfqError) as e:
        d.load("/nonexistent/graph.txt")
    assert e.value.name == "EIO"


def test_pick_sources():
    g = d.gen_rmat(12, 8, seed=1)
    s = g.pick_sources(64, seed=4)
    assert len(set(s.tolist())) == 64
    assert np.all(g.degrees()[s] > 0)
    assert np.array_equal(s, g.pick_sources(64, seed=4))


# ---------------------------------------------------------------- parallel host I/O
@pytest.fixture
def host_threads():
    yield d.set_host_threads
    d.set_host_threads(0)


@pytest.mark.parametrize("fmt", ["snap", "dat"])
def test_parallel_text_io_matches_serial(tmp_path, fmt, host_threads):
    """Text written and parsed over 2..13 pieces is byte- and CSR-identical to
    the one-thread result, with and without builder flags."""
    g = d.gen_rmat(11, 8, seed=5)
    g.source = 7
    host_threads(1)
    g.save(tmp_path / "one", fmt)
    ref = d.load(tmp_path / "one")
    flags = d.CSR_SYMMETRIZE | d.CSR_DEDUP | d.CSR_NO_SELF_LOOPS
    ref_f = d.load(tmp_path / "one", flags=flags)
    one = (tmp_path / "one").read_bytes()
    assert np.array_equal(ref.offsets, g.offsets) and np.array_equal(ref.cols, g.cols)
    for t in (2, 3, 8, 13):
        host_threads(t)
        assert d.host_threads() == t
        g.save(tmp_path / f"t{t}", fmt)
        assert (tmp_path / f"t{t}").read_bytes() == one
        h = d.load(tmp_path / f"t{t}")
        assert np.array_equal(h.offsets, ref.offsets) and np.array_equal(h.cols, ref.cols)
        assert h.source == (7 if fmt == "dat" else 0)
        hf = d.load(tmp_path / f"t{t}", flags=flags)
        assert np.array_equal(hf.offsets, ref_f.offsets) and np.array_equal(hf.cols, ref_f.cols)


def test_parallel_csr_builder_is_stable(host_threads):
    """The chunked counting sort keeps input order within each row (no DEDUP),
    so every thread count gives the serial CSR."""
    rng = np.random.default_rng(3)
    m, n = 20000, 300
    src = rng.integers(0, n, m, dtype=np.int32)
    dst = rng.integers(0, n, m, dtype=np.int32)
    for flags in (0, d.CSR_SYMMETRIZE, d.CSR_NO_SELF_LOOPS | d.CSR_SYMMETRIZE, d.CSR_DEDUP | d.CSR_SYMMETRIZE):
        host_threads(1)
        a = d.from_edges(src, dst, n, flags)
        for t in (2, 5, 16):
            host_threads(t)
            b = d.from_edges(src, dst, n, flags)
            assert np.array_equal(a.offsets, b.offsets) and np.array_equal(a.cols, b.cols), (flags, t)
    # the serial definition: row u lists, in input order, v for every u->v
    host_threads(7)
    c = d.from_edges(src, dst, n)
    for u in (0, 17, 299):
        assert c.cols[c.offsets[u]:c.offsets[u + 1]].tolist() == dst[src == u].tolist()


def _edge_lines(k):
    return "".join(f"{i % 97}\t{(i * 7) % 101}\n" for i in range(k))


@pytest.mark.parametrize("body,expect", [
    (_edge_lines(300) + "12 x\n" + _edge_lines(400), "edge line 301 is not"),
    (_edge_lines(700) + "5 4294967296\n" + _edge_lines(10), "edge line 701 has id out of int32 range"),
    ("# c\n" + _edge_lines(50) + "# Nodes: 9 Edges: 1\n" + _edge_lines(50) + "7\n", "edge line 101 is not"),
])
def test_parallel_snap_errors_name_the_serial_line(tmp_path, body, expect, host_threads):
    p = tmp_path / "bad.txt"
    p.write_text("# Nodes: 200 Edges: 10\n" + body)
    msgs = set()
    for t in (1, 3, 11):
        host_threads(t)
        with pytest.raises(d.DfqError) as e:
            d.load(p)
        assert e.value.name == "EFORMAT" and expect in str(e.value)
        msgs.add(str(e.value))
    assert len(msgs) == 1


def _dat(n, e, nodes, edges):
    return f"{n} {e} 0\n" + "".join(f"{a} {b}\n" for a, b in nodes) + "".join(f"{a} {b}\n" for a, b in edges)


@pytest.mark.parametrize("which,expect", [
    ("node_malformed", "node record 50 missing or malformed"),
    ("node_range", "node 100 has start=0 length=999999"),
    ("edge_range", "edge 400 targets 5000 outside [0,200)"),
    ("edge_malformed", "edge record 401 missing or malformed"),
    ("truncated", "edge record 999 missing or malformed"),
    ("truncated_nodes", "node record 150 missing or malformed"),
])
def test_parallel_dat_errors_name_the_serial_record(tmp_path, which, expect, host_threads):
    n, e = 200, 1000
    nodes = [(5 * i, 5) for i in range(n)]
    edges = [((i * 13) % n, 1) for i in range(e)]
    if which == "node_malformed":
        nodes[50] = ("1z", 5)
        nodes[120] = (0, 999999)  # a later error must not win
    if which == "node_range":
        nodes[100] = (0, 999999)
        edges[3] = (5000, 1)
    if which == "edge_range":
        edges[400] = (5000, 1)
        edges[700] = ("q", 1)
    if which == "edge_malformed":
        edges[401] = (3, "1.5")
    text = _dat(n, e, nodes, edges)
    if which == "truncated":
        text = text[: text.rstrip("\n").rfind("\n") + 1]
    if which == "truncated_nodes":
        text = f"{n} {e} 0\n" + "".join(f"{a} {b}\n" for a, b in nodes[:150])
    p = tmp_path / "bad.dat"
    p.write_text(text)
    msgs = set()
    for t in (1, 4, 9):
        host_threads(t)
        with pytest.raises(d.DfqError) as ex:
            d.load(p)
        assert ex.value.name == "EFORMAT" and expect in str(ex.value), str(ex.value)
        msgs.add(str(ex.value))
    assert len(msgs) == 1


def test_set_host_threads_bounds():
    with pytest.raises(d.DfqError):
        d.set_host_threads(-1)
    with pytest.raises(d.DfqError):
        d.set_host_threads(1000)
    d.set_host_threads(0)
    assert d.host_threads() >= 1
