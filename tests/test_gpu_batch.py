"""Graph pools and batched BFS: many (graph, source)
queries in one persistent launch, wide queries on the whole grid and narrow
ones one per block; every result bit-exact against the oracle, with and
without CUDA-graph capture and replay, with parents, and per-query plain
launches through the same pool."""
import numpy as np
import pytest

import dfqbfs as d
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def mixed_graphs():
    gs = [d.gen_rmat(s, ef, seed=100 + s) for s, ef in [(8, 8), (10, 16), (12, 8), (13, 16), (14, 32)]]
    gs += [d.gen_grid(side, 0.02, seed=side)[0] for side in (16, 48, 100, 160)]
    gs += [d.gen_zipf_geometric(5000, 4.7, 2.1, seed=3), d.from_edges([], [], 7)]
    return gs


def opts_small_wide():
    o = d.default_opts()
    o.wide_min_edges = 100_000   # the larger RMAT graphs run on the whole grid
    o.wide_min_degree = 8
    return o


def make_queries(torch, graphs, per_graph=3, seed=0, parents=False):
    rng = np.random.default_rng(seed)
    qs, meta = [], []
    for gi, g in enumerate(graphs):
        for k in range(per_graph):
            src = int(rng.integers(0, g.n))
            lv = torch.full((g.n,), -7, dtype=torch.int32, device="cuda")
            pa = torch.full((g.n,), -7, dtype=torch.int32, device="cuda") if parents else None
            qs.append((gi, src, lv, pa))
            meta.append((g, src))
    rng.shuffle(qs := list(zip(qs, meta)))
    return [q for q, _ in qs], [m for _, m in qs]


def check_results(qs, meta, res, parents=False):
    for (gi, src, lv, pa), (g, s), r in zip(qs, meta, res):
        want = oracle.bfs(g.offsets, g.cols, s)
        got = lv.cpu().numpy()
        assert oracle.compare(want, got)["mismatches"] == 0, (gi, s)
        assert r.status == 0 and r.edges == oracle.reached_edges(g.offsets, want) and r.reached == (want >= 0).sum()
        assert r.end_us >= r.start_us >= 0
        if parents:
            assert oracle.validate_tree(g.offsets, g.cols, s, got, pa.cpu().numpy()) == 0


@pytest.mark.parametrize("flags", [0, d.BATCH_GRAPH])
def test_batch_mixed_pool(torch, flags):
    graphs = mixed_graphs()
    with d.Pool(graphs, opts_small_wide()) as pool:
        assert any(pool.info(i)[2] for i in range(len(graphs)))       # some wide
        assert not all(pool.info(i)[2] for i in range(len(graphs)))   # some narrow
        qs, meta = make_queries(torch, graphs, 3, seed=1)
        res, ms = pool.batch(qs, flags)
        assert ms > 0 and sum(r.wide for r in res) > 0
        check_results(qs, meta, res)
        # second run with new sources: a captured graph is replayed with new table contents
        qs2, meta2 = make_queries(torch, graphs, 3, seed=2)
        res2, _ = pool.batch(qs2, flags)
        check_results(qs2, meta2, res2)


def test_batch_with_parents(torch):
    graphs = mixed_graphs()[:7]
    with d.Pool(graphs, opts_small_wide()) as pool:
        qs, meta = make_queries(torch, graphs, 2, seed=3, parents=True)
        res, _ = pool.batch(qs, d.BATCH_GRAPH)
        check_results(qs, meta, res, parents=True)


@pytest.mark.parametrize("flags", [0, d.BATCH_GRAPH])
def test_batch_with_hot_cache(torch, flags):
    """The shared hot-vertex cache in both group shapes (whole grid and one
    block), with parents: same levels, valid trees."""
    graphs = mixed_graphs()
    o = opts_small_wide()
    o.hot_cache = 32  # 32 KB: the visited bits of the first 262,144 ids
    with d.Pool(graphs, o) as pool:
        qs, meta = make_queries(torch, graphs, 2, seed=5, parents=True)
        res, _ = pool.batch(qs, flags)
        check_results(qs, meta, res, parents=True)
        for gi, g in enumerate(graphs[:4]):
            lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
            pool.bfs(gi, 0, lv)
            assert np.array_equal(lv.cpu().numpy(), oracle.bfs(g.offsets, g.cols, 0))


def test_batch_all_narrow_and_all_wide(torch):
    graphs = [d.gen_rmat(11, 16, seed=7), d.gen_grid(64, 0.0, seed=1)[0]]
    for wide_edges in (1 << 30, 1):
        o = d.default_opts()
        o.wide_min_edges = wide_edges
        o.wide_min_degree = 1
        with d.Pool(graphs, o) as pool:
            qs, meta = make_queries(torch, graphs, 4, seed=4)
            res, _ = pool.batch(qs)
            check_results(qs, meta, res)
            assert all(r.wide == (wide_edges == 1) for r in res)


def test_pool_single_launches_match(torch):
    graphs = mixed_graphs()
    with d.Pool(graphs, opts_small_wide()) as pool:
        for gi, g in enumerate(graphs):
            src = int(np.random.default_rng(gi).integers(0, g.n))
            lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
            st = pool.bfs(gi, src, lv)
            want = oracle.bfs(g.offsets, g.cols, src)
            assert np.array_equal(lv.cpu().numpy(), want)
            assert st.edges == oracle.reached_edges(g.offsets, want)


def test_batch_rejects_bad_queries(torch):
    graphs = mixed_graphs()[:3]
    with d.Pool(graphs) as pool:
        lv = torch.empty(graphs[0].n, dtype=torch.int32, device="cuda")
        pa = torch.empty(graphs[0].n, dtype=torch.int32, device="cuda")
        with pytest.raises(d.DfqError) as e:
            pool.batch([(0, 0, lv, pa), (0, 1, lv)])
        assert e.value.name == "EINVAL"
        with pytest.raises(d.DfqError):
            pool.batch([(len(graphs), 0, lv)])
        with pytest.raises(d.DfqError):
            pool.batch([(0, graphs[0].n, lv)])


def test_renumbered_wide_graphs(torch):
    """Wide graphs with skewed degrees are stored hub-first in the pool; batch,
    single launch and server still answer in input ids (levels, trees, E_R)."""
    graphs = [d.gen_rmat(17, 16, seed=41), d.gen_grid(40, 0.02, seed=41)[0], d.gen_rmat(10, 8, seed=42)]
    o = d.default_opts()
    o.wide_min_edges = 1 << 20
    with d.Pool(graphs, o) as pool:
        assert pool.info(0)[2] and not pool.info(1)[2]
        for parents in (False, True):
            qs, meta = make_queries(torch, graphs, 3, seed=43, parents=parents)
            res, _ = pool.batch(qs, d.BATCH_GRAPH)
            check_results(qs, meta, res, parents=parents)
        g = graphs[0]
        for s in g.pick_sources(2, seed=44):
            lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
            pa = torch.empty(g.n, dtype=torch.int32, device="cuda")
            pool.bfs(0, int(s), lv, pa)
            want = oracle.bfs(g.offsets, g.cols, int(s))
            assert np.array_equal(lv.cpu().numpy(), want)
            assert oracle.validate_tree(g.offsets, g.cols, int(s), lv.cpu().numpy(), pa.cpu().numpy()) == 0
        with d.Server(pool, with_parents=True) as srv:
            ids = {srv.submit(0, int(s)): int(s) for s in g.pick_sources(3, seed=45)}
            done = srv.drain(60.0)
            assert {r.id for r in done} == set(ids) and all(r.status == 0 for r in done)
            for rid, s in ids.items():
                lv, pa = srv.levels(rid, g.n, parents=True)
                want = oracle.bfs(g.offsets, g.cols, s)
                assert np.array_equal(lv, want)
                assert oracle.validate_tree(g.offsets, g.cols, s, lv, pa) == 0
                srv.release(rid)


def test_pool_autotune_and_set_opts(torch):
    """The batch kernel tuned on the pool itself: the winner is installed,
    a captured batch is re-captured after an option change, results stay
    exact; options fixed at pool creation are refused."""
    graphs = mixed_graphs()
    with d.Pool(graphs, opts_small_wide()) as pool:
        qs, meta = make_queries(torch, graphs, 2, seed=9)
        res, _ = pool.batch(qs, d.BATCH_GRAPH)
        check_results(qs, meta, res)
        best = pool.autotune(qs)
        assert pool.opts().as_dict() == best.as_dict()
        res, _ = pool.batch(qs, d.BATCH_GRAPH)
        check_results(qs, meta, res)
        o = pool.opts()
        o.block_threads = 1024 if o.block_threads != 1024 else 512
        pool.set_opts(o)
        res, _ = pool.batch(qs, d.BATCH_GRAPH)
        check_results(qs, meta, res)
        bad = pool.opts()
        bad.wide_min_edges = bad.wide_min_edges * 2
        with pytest.raises(d.DfqError):
            pool.set_opts(bad)


@pytest.mark.parametrize("flags", [0, d.BATCH_GRAPH])
@pytest.mark.parametrize("parents", [False, True])
def test_batch_gangs_for_high_diameter_graphs(torch, flags, parents):
    """Large high-diameter graphs (grids of >= 65,536 vertices) run on gangs
    of blocks: few such queries get large gangs, many get small ones, and
    with more queries than gang blocks they fall back to one block each.
    Every result stays exact, in every mix with wide and narrow queries."""
    grids = [d.gen_grid(side, 0.02, seed=side)[0] for side in (260, 300, 400)]
    graphs = grids + [d.gen_rmat(16, 16, seed=5), d.gen_rmat(11, 8, seed=6), d.gen_grid(40, 0.0, seed=1)[0]]
    o = opts_small_wide()
    with d.Pool(graphs, o) as pool:
        for per_graph in (1, 3, 40):  # 3 / 9 / 120 gang queries
            qs, meta = make_queries(torch, graphs if per_graph < 40 else graphs[:3], per_graph, seed=per_graph,
                                    parents=parents)
            res, _ = pool.batch(qs, flags)
            check_results(qs, meta, res, parents=parents)
            res, _ = pool.batch(qs, flags)  # a replay of the same shape
            check_results(qs, meta, res, parents=parents)
