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
