"""Serving: continuous batching on the device.

Requests are submitted while others run; each result must be the same alone
and in the mix - bit-exact levels (and valid parent trees) against the
oracle, equal to a request served on its own.  Also covered: admission under
a small HBM budget (requests wait for arena space), a narrow request that
outgrows its block's queues and is rerun on the whole grid, and the serving
kernel leaving when idle and being relaunched."""
import time

import numpy as np
import pytest

import dfqbfs as d
import oracle

pytestmark = pytest.mark.gpu


def pool_graphs():
    gs = [d.gen_rmat(s, ef, seed=200 + s) for s, ef in [(9, 8), (11, 16), (13, 16), (15, 16)]]
    gs += [d.gen_grid(side, 0.02, seed=side)[0] for side in (20, 64, 128)]
    gs += [d.gen_zipf_geometric(3000, 4.7, 2.1, seed=5)]
    return gs


def pool_opts():
    o = d.default_opts()
    o.wide_min_edges = 200_000  # R-MAT 13 and 15 are served by the whole grid
    o.wide_min_degree = 8
    return o


def requests(graphs, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        gi = int(rng.integers(0, len(graphs)))
        out.append((gi, int(rng.integers(0, graphs[gi].n))))
    return out


def check(server, graphs, reqs, results, parents=False):
    by_id = {r.id: r for r in results}
    assert len(by_id) == len(reqs)
    for rid, (gi, s) in reqs.items():
        r = by_id[rid]
        g = graphs[gi]
        assert r.status == 0, r.status
        lv, pa = server.levels(rid, g.n, parents)
        want = oracle.bfs(g.offsets, g.cols, s)
        assert np.array_equal(lv, want), (gi, s)
        assert r.edges == oracle.reached_edges(g.offsets, want) and r.reached == (want >= 0).sum()
        if parents:
            assert oracle.validate_tree(g.offsets, g.cols, s, lv, pa) == 0
        server.release(rid)


def test_same_alone_and_in_the_mix():
    graphs = pool_graphs()
    with d.Pool(graphs, pool_opts()) as pool, d.Server(pool, idle_ms=50) as srv:
        # alone: one request at a time
        pairs = requests(graphs, 12, seed=1)
        alone = {}
        for gi, s in pairs:
            rid = srv.submit(gi, s)
            res = srv.drain()
            assert len(res) == 1 and res[0].id == rid and res[0].status == 0
            alone[(gi, s)] = srv.levels(rid, graphs[gi].n)[0]
            srv.release(rid)
        # in the mix: the same pairs inside a stream submitted while earlier
        # requests are on the device
        stream = requests(graphs, 300, seed=2)
        for k, pair in enumerate(pairs):
            stream.insert(25 * k + 7, pair)
        mix, results = {}, []
        for k, (gi, s) in enumerate(stream):
            mix[srv.submit(gi, s, tag=k)] = (gi, s)
            if k % 7 == 0:
                results += srv.poll()
        results += srv.drain()
        assert any(r.wide for r in results) and not all(r.wide for r in results)
        for r in results:
            pair = mix[r.id]
            if pair in alone:
                assert np.array_equal(srv.levels(r.id, graphs[pair[0]].n)[0], alone[pair])
        check(srv, graphs, mix, results)


def test_admission_waits_for_hbm_budget():
    graphs = pool_graphs()
    biggest = max(g.n for g in graphs)
    with d.Pool(graphs, pool_opts()) as pool, d.Server(pool, hbm_budget_bytes=4 * biggest * 3, idle_ms=50) as srv:
        reqs = {srv.submit(gi, s): (gi, s) for gi, s in requests(graphs, 60, seed=3)}
        results, t0 = [], time.time()
        while srv.pending:
            assert time.time() - t0 < 60, f"{srv.pending} requests still pending"
            got = srv.poll()
            results += got
            for r in got:  # free arena space as results are consumed
                gi, s = reqs[r.id]
                lv, _ = srv.levels(r.id, graphs[gi].n)
                assert np.array_equal(lv, oracle.bfs(graphs[gi].offsets, graphs[gi].cols, s))
                srv.release(r.id)
        assert len(results) == 60 and all(r.status == 0 for r in results)


def test_narrow_overflow_rerun_on_grid():
    # 600^2 grid: BFS frontiers reach ~600 (corner) and ~1200 (centre) vertices,
    # far beyond a block's 256 shared slots plus 64 overflow slots
    graphs = [d.gen_grid(600, 0.0, seed=1)[0]]
    o = pool_opts()
    with d.Pool(graphs, o) as pool, d.Server(pool, narrow_queue_cap=64, idle_ms=50) as srv:
        reqs = {srv.submit(0, s): (0, s) for s in (0, 300 * 600 + 300)}
        results = srv.drain()
        assert all(r.retried for r in results)
        check(srv, graphs, reqs, results)


def test_parents_and_idle_relaunch():
    graphs = pool_graphs()
    with d.Pool(graphs, pool_opts()) as pool, d.Server(pool, with_parents=True, idle_ms=5) as srv:
        for round_ in range(3):
            reqs = {srv.submit(gi, s): (gi, s) for gi, s in requests(graphs, 40, seed=10 + round_)}
            results = srv.drain()
            check(srv, graphs, reqs, results, parents=True)
            time.sleep(0.05)  # longer than idle_ms: the serving kernel leaves and is relaunched
