"""The CPU oracle (CPU only): hand-built cases, C vs pure-Python restatement,
validators, and the golden levels produced by the reference's own kernel."""
from pathlib import Path

import numpy as np
import pytest

import dfqbfs as d
import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


def csr(n, edges):
    s = [u for u, _ in edges]
    t = [v for _, v in edges]
    return d.from_edges(s, t, n)


HAND = {
    # name: (n, edges, src, expected levels)
    "path": (5, [(0, 1), (1, 2), (2, 3), (3, 4)], 0, [0, 1, 2, 3, 4]),
    "path_mid": (5, [(0, 1), (1, 2), (2, 3), (3, 4)], 2, [-1, -1, 0, 1, 2]),
    "star": (6, [(0, i) for i in range(1, 6)], 0, [0, 1, 1, 1, 1, 1]),
    "two_components": (6, [(0, 1), (1, 2), (3, 4), (4, 5)], 0, [0, 1, 2, -1, -1, -1]),
    "isolated_source": (4, [(1, 2), (2, 3)], 0, [0, -1, -1, -1]),
    "self_loop": (3, [(0, 0), (0, 1), (1, 1), (1, 2)], 0, [0, 1, 2]),
    "duplicates": (3, [(0, 1), (0, 1), (1, 2), (1, 2), (0, 2)], 0, [0, 1, 1]),
    "degree_zero_mid": (4, [(0, 1), (0, 2), (2, 3)], 0, [0, 1, 1, 2]),
    "diamond": (4, [(0, 1), (0, 2), (1, 3), (2, 3)], 0, [0, 1, 1, 2]),
    "back_edges": (4, [(0, 1), (1, 0), (1, 2), (2, 0), (2, 3)], 0, [0, 1, 2, 3]),
}


@pytest.mark.parametrize("name", sorted(HAND))
def test_hand_cases(name):
    n, edges, src, want = HAND[name]
    g = csr(n, edges)
    assert oracle.bfs(g.offsets, g.cols, src).tolist() == want
    assert oracle.py_bfs(g.offsets.tolist(), g.cols.tolist(), src) == want


@pytest.mark.parametrize("seed", range(20))
def test_c_matches_python(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 300))
    m = int(rng.integers(0, 4 * n))
    g = d.from_edges(rng.integers(0, n, m), rng.integers(0, n, m), n)
    src = int(rng.integers(0, n))
    a = oracle.bfs(g.offsets, g.cols, src)
    b = oracle.py_bfs(g.offsets.tolist(), g.cols.tolist(), src)
    assert a.tolist() == b


def test_compare_semantics():
    want = np.array([0, 1, 2, -1, -1], np.int32)
    assert oracle.compare(want, want)["mismatches"] == 0
    r = oracle.compare(want, np.array([0, 1, 3, -1, 1], np.int32))
    assert r["near_nodes"] == 3 and r["near_errors"] == 1 and r["extra"] == 1 and r["dist"] == 1
    # the reference rule alone (near_errors) misses the extra vertex
    assert r["mismatches"] == 2


def test_tree_validator_rejects_corruption():
    g = d.gen_rmat(10, 8, seed=1)
    src = int(g.pick_sources(1, seed=1)[0])
    lv = oracle.bfs(g.offsets, g.cols, src)
    # build a valid parent array from the levels
    par = np.full(g.n, -1, np.int32)
    par[src] = src
    for u in range(g.n):
        for v in g.cols[g.offsets[u]:g.offsets[u + 1]]:
            if lv[u] >= 0 and lv[v] == lv[u] + 1 and par[v] < 0:
                par[v] = u
    assert oracle.validate_tree(g.offsets, g.cols, src, lv, par) == 0
    reached = np.flatnonzero((lv > 0))
    v = int(reached[len(reached) // 2])
    bad = par.copy(); bad[v] = src if lv[v] != 1 else -1  # wrong level span or missing
    assert oracle.validate_tree(g.offsets, g.cols, src, lv, bad) != 0
    bad = par.copy(); bad[src] = -1
    assert oracle.validate_tree(g.offsets, g.cols, src, lv, bad) != 0
    unreached = np.flatnonzero(lv < 0)
    if len(unreached):
        bad = par.copy(); bad[unreached[0]] = src
        assert oracle.validate_tree(g.offsets, g.cols, src, lv, bad) != 0
    # a parent one level up but with no edge to the child
    lv1 = np.flatnonzero(lv == 2)
    if len(lv1):
        w = int(lv1[0])
        cands = [u for u in np.flatnonzero(lv == 1) if w not in g.cols[g.offsets[u]:g.offsets[u + 1]]]
        if cands:
            bad = par.copy(); bad[w] = cands[0]
            assert oracle.validate_tree(g.offsets, g.cols, src, lv, bad) == 1 + w


def test_reached_edges():
    g = csr(5, [(0, 1), (0, 2), (1, 2), (3, 4)])
    lv = oracle.bfs(g.offsets, g.cols, 0)
    assert oracle.reached_edges(g.offsets, lv) == 3


def golden_files():
    return sorted(GOLDEN.glob("ref_*.npz"))


def test_golden_fixtures_present():
    assert golden_files(), "reference golden fixtures are missing from tests/golden"


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.stem)
def test_oracle_matches_reference_golden(path):
    """Levels produced by the reference's own kernel on the GPU (see
    tests/golden/make_golden.py) equal the oracle's, vertex for vertex."""
    z = np.load(path)
    for k, src in enumerate(z["sources"]):
        want = z["levels"][k]
        got = oracle.bfs(z["offsets"], z["cols"], int(src))
        assert np.array_equal(got, want), f"{path.name} source {src}"
