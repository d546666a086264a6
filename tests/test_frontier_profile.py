"""dfq_frontier_profile (CPU): the idle-lane and bin counts of the
reference's frontier profiler (design/shared-q/atomic-sa/our-sep/upper-bound/
bfs_ftr_prof.cu:129-140), computed on the host from oracle levels, equal a
direct restatement of the reference's per-vertex formula, for any number of
host threads."""
import numpy as np
import pytest

import dfqbfs as d
import oracle


def brute(offsets, levels, tiles, threads):
    depth = int(levels.max())
    idle = np.zeros((depth + 1, 5), np.int64)
    cnt = np.zeros((depth + 1, 5), np.int64)
    deg = np.diff(offsets.astype(np.int64))
    for v in range(len(levels)):
        lv, dd = int(levels[v]), int(deg[v])
        if lv < 0 or dd == 0:
            continue
        b = next((i for i in range(4) if dd <= tiles[i]), 4)
        idle[lv, b] += tiles[b] - (dd & (tiles[b] - 1)) if b < 4 else threads - dd % threads
        cnt[lv, b] += 1
    return idle, cnt


@pytest.mark.parametrize("tiles,threads", [((16, 128, 1024, 8192), 304 * 1024), ((8, 64, 1024, 16384), 72 * 1024),
                                           ((2, 4, 8, 16), 100)])
def test_matches_reference_formula(tiles, threads):
    for g, src in [(d.gen_rmat(12, 16, seed=4), None), (d.gen_zipf_geometric(20000, 4.7, 2.1, seed=4), 0),
                   (d.gen_grid(40, 0.05, seed=4)[0], 0)]:
        s = int(g.pick_sources(1, seed=4)[0]) if src is None else src
        lv = oracle.bfs(g.offsets, g.cols, s)
        idle, cnt = d.frontier_profile(g, lv, tiles, threads)
        want_idle, want_cnt = brute(g.offsets, lv, tiles, threads)
        assert np.array_equal(idle, want_idle) and np.array_equal(cnt, want_cnt)
        # every reached vertex with edges is counted once, in its own level
        deg = np.diff(g.offsets)
        assert cnt.sum() == int(((lv >= 0) & (deg > 0)).sum())


def test_quirks_limits_and_threads():
    # a degree equal to a tile is charged a whole tile, as in the reference
    g = d.from_edges([0] * 16 + [1], list(range(1, 17)) + [0], 17, 0)
    lv = oracle.bfs(g.offsets, g.cols, 0)
    idle, cnt = d.frontier_profile(g, lv, (16, 128, 1024, 8192), 1024)
    assert cnt[0, 0] == 1 and idle[0, 0] == 16
    # max_levels caps the rows; host thread count never changes the sums
    big = d.gen_rmat(15, 8, seed=6)
    lv = oracle.bfs(big.offsets, big.cols, int(big.pick_sources(1, seed=6)[0]))
    full = d.frontier_profile(big, lv)
    two, _ = d.frontier_profile(big, lv, max_levels=2)
    assert np.array_equal(two, full[0][:2])
    prev = d.host_threads()
    try:
        d.set_host_threads(1)
        one = d.frontier_profile(big, lv)
    finally:
        d.set_host_threads(prev)
    assert np.array_equal(one[0], full[0]) and np.array_equal(one[1], full[1])
    with pytest.raises(d.DfqError):
        d.frontier_profile(big, lv, (16, 100, 1024, 8192))   # not a power of two
    with pytest.raises(d.DfqError):
        d.frontier_profile(big, lv, (128, 16, 1024, 8192))   # not increasing
    with pytest.raises(d.DfqError):
        d.frontier_profile(big, lv, threads=0)


def test_null_arguments_and_empty_graph():
    import ctypes as C
    L = d.lib()
    tiles = (C.c_int32 * 4)(16, 128, 1024, 8192)
    assert L.dfq_frontier_profile(None, None, tiles, 1024, 4, None, None) == -1
    g = d.gen_rmat(8, 4, seed=1)
    c = g._as_c()
    assert L.dfq_frontier_profile(C.byref(c), None, tiles, 1024, 4, None, None) == -1
    lv = np.full(g.n, -1, np.int32)  # nothing reached: no levels
    idle, cnt = d.frontier_profile(g, lv)
    assert idle.shape == (0, 5) and cnt.shape == (0, 5)
    with pytest.raises(ValueError):
        d.frontier_profile(g, lv[:-1])
