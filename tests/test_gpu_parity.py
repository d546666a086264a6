"""GPU parity: levels from the DFQ kernel (through the C ABI) equal the CPU
oracle bit for bit; parents form a BFS tree; statistics match E_R.

Covers the bins and queues of the kernel: degrees on every bin boundary,
forced shared-queue overflow, the large bin with and without TMA staging,
every block size, host and device output buffers, repeated runs, and the
full-size configurations through size-independent properties."""
import numpy as np
import pytest

import dfqbfs as d
import oracle

pytestmark = pytest.mark.gpu


def run_and_check(g, src, opts=None, parents=True, graph=None):
    own = graph is None
    dg = graph or d.Graph(g, opts=opts)
    try:
        if opts is not None and not own:
            dg.set_opts(opts)
        lv, pa, st = dg.bfs(src, parents=parents)
    finally:
        if own:
            dg.close()
    want = oracle.bfs(g.offsets, g.cols, src)
    cmp = oracle.compare(want, lv)
    assert cmp["mismatches"] == 0, cmp
    if parents:
        bad = oracle.validate_tree(g.offsets, g.cols, src, lv, pa)
        assert bad == 0, f"parent tree invalid at vertex {bad - 1}"
    assert st.edges == oracle.reached_edges(g.offsets, want)
    assert st.reached == int((want >= 0).sum())
    assert st.depth == int(want.max())
    return lv, st


def opts(**kw):
    o = d.default_opts()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


@pytest.fixture(scope="module")
def c1():
    return d.gen_zipf_geometric(262144, 4.7, 2.1, seed=1)


def test_config1_zipf_geometric_source0(c1):
    run_and_check(c1, 0)


@pytest.mark.parametrize("seed", range(60))
def test_random_small_graphs(seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(1, 4097))
    kind = seed % 3
    if kind == 0:  # uniform random directed
        m = int(rng.integers(0, 8 * n + 1))
        g = d.from_edges(rng.integers(0, n, m), rng.integers(0, n, m), n)
    elif kind == 1:  # a few hubs with degrees across the bin boundaries
        src, dst = [], []
        for h in range(min(n, 6)):
            k = int(min(n, rng.choice([8, 9, 31, 32, 33, 64, 65, 1023, 1024, 1025, 2048, 4096])))
            src += [h] * k
            dst += rng.choice(n, size=k, replace=False).tolist()
        m = 3 * n
        src += rng.integers(0, n, m).tolist()
        dst += rng.integers(0, n, m).tolist()
        g = d.from_edges(src, dst, n, d.CSR_SYMMETRIZE | d.CSR_DEDUP)
    else:
        side = max(1, int(np.sqrt(n)))
        g, _ = d.gen_grid(side, float(rng.uniform(0, 0.3)), seed=seed)
    src = int(rng.integers(0, g.n))
    run_and_check(g, src)


BOUNDARY_DEGS = [1, 2, 3, 4, 5, 7, 8, 9, 31, 32, 33, 63, 64, 65, 127, 128, 1023, 1024, 1025, 2047, 2048,
                 2049, 4095, 4096, 4097, 16384, 16385]


@pytest.fixture(scope="module")
def boundary_graph():
    rng = np.random.default_rng(7)
    n = 40000
    src, dst = [], []
    for i, k in enumerate(BOUNDARY_DEGS):
        src += [i] * k
        dst += rng.choice(n, size=k, replace=False).tolist()
    # chain the hubs so one BFS reaches all of them at different levels
    src += list(range(len(BOUNDARY_DEGS) - 1))
    dst += list(range(1, len(BOUNDARY_DEGS)))
    m = 60000
    src += rng.integers(0, n, m).tolist()
    dst += rng.integers(0, n, m).tolist()
    return d.from_edges(src, dst, n, d.CSR_DEDUP)


@pytest.mark.parametrize("B", [256, 512, 1024])
@pytest.mark.parametrize("tma", [0, 1])
@pytest.mark.parametrize("probe", [0, 1])
def test_boundaries_all_block_sizes(boundary_graph, B, tma, probe):
    run_and_check(boundary_graph, 0, opts(block_threads=B, use_tma=tma, probe_first=probe))


@pytest.mark.parametrize("medium,large,piece,budget", [
    (1, 32, 64, 8192),              # everything medium or large, tiny pieces
    (1 << 30, 1 << 30, 256, 8192),  # no medium, no large: all warp-gathered
    (8, 64, 128, 64),
    (32, 1024, 512, 1 << 30),       # unlimited local edge budget
    (64, 16384, 1024, 1),           # every warp batch overflows to the global queue
])
def test_bin_thresholds(boundary_graph, medium, large, piece, budget):
    run_and_check(boundary_graph, 0, opts(medium_min_degree=medium, large_min_degree=large, piece_edges=piece,
                                          local_edge_budget=budget))


@pytest.mark.parametrize("cap", [1, 16, 100])
def test_forced_overflow(cap):
    g = d.gen_rmat(14, 16, seed=3)
    src = int(g.pick_sources(1, seed=3)[0])
    _, st = run_and_check(g, src, opts(local_queue_cap=cap))
    assert st.overflow > 0


def test_large_bin_used():
    g = d.gen_rmat(16, 16, seed=4)
    src = int(g.pick_sources(1, seed=4)[0])
    _, st = run_and_check(g, src, opts(large_min_degree=256, piece_edges=64))
    assert st.large > 0


def test_grid_high_diameter():
    g, _ = d.gen_grid(512, 0.01, seed=5)
    lv, st = run_and_check(g, 0)
    assert st.depth > 1000


def test_rmat18_several_sources():
    g = d.gen_rmat(18, 16, seed=6)
    with d.Graph(g) as dg:
        for s in g.pick_sources(4, seed=6):
            run_and_check(g, int(s), graph=dg)


@pytest.mark.parametrize("kind", ["rmat", "grid"])
def test_level_profile_matches_oracle(kind):
    """The per-level profile counts what the oracle's levels imply: level L
    expands the vertices at depth L with out-degree > 0 and scans their
    degree sum; device clock readings are ordered."""
    if kind == "rmat":
        g = d.gen_rmat(16, 16, seed=12)
        src = int(g.pick_sources(1, seed=12)[0])
    else:
        g, _ = d.gen_grid(128, 0.01, seed=12)
        src = 0
    want = oracle.bfs(g.offsets, g.cols, src)
    deg = g.degrees()
    with d.Graph(g, opts=opts(profile=1)) as dg:
        dg.bfs(src)
        st = dg.last_stats()
        prof = dg.last_levels(64)
        ns, fr = dg.last_trace(64)
    assert len(prof) == min(64, st.levels + 1) and len(ns) == len(prof)
    for L, row in enumerate(prof):
        at = (want == L) & (deg > 0)
        assert row["frontier"] == int(at.sum()) == fr[L], L
        if L < st.levels:
            assert row["edges"] == int(deg[at].sum()), L
            assert 0 <= row["overflow"] <= row["frontier"]
            assert row["probe"] in (0, 1)
            # blocks with nothing to do can finish before block 0 stamps the start
            assert row["us_work"] >= 0 and row["us_spread"] >= 0
            if "us_barrier" in row:
                assert row["us_barrier"] >= 0
    if st.levels < 64:
        assert sum(r["edges"] for r in prof) == st.edges
    assert np.all(np.diff(ns) >= 0)


@pytest.mark.parametrize("order,hot,block", [(1, 0, 512), (2, 0, 512), (2, -1, 512), (1, 32, 512), (2, 32, 512),
                                             (2, 8, 512), (2, 32, 1024), (1, 32, 256)])
def test_vertex_order_and_hot_cache(order, hot, block):
    """Hub-first relabelling and the shared hot-vertex cache change only how
    the kernel works: levels, parents (in input ids) and E_R stay exact, on
    the whole grid and in a small graph that the cache covers entirely."""
    for g, srcs in [(d.gen_rmat(16, 16, seed=21), None), (d.gen_zipf_geometric(50000, 4.7, 2.1, seed=21), [0, 7])]:
        srcs = srcs or [int(x) for x in g.pick_sources(3, seed=21)]
        with d.Graph(g, opts=opts(vertex_order=order, hot_cache=hot, block_threads=block)) as dg:
            for s in srcs:
                run_and_check(g, int(s), graph=dg)
                run_and_check(g, int(s), graph=dg, parents=False)


@pytest.mark.parametrize("block", [256, 512, 1024])
@pytest.mark.parametrize("tma", [0, 1])
def test_hot_cache_bin_boundaries(block, tma):
    """The hot-vertex cache on a hub graph whose degrees sit on every bin
    boundary (small gather, medium warp lists, large pieces), hub-first ids
    forced so the cache holds the hubs: bit-exact levels, valid parents."""
    rng = np.random.default_rng(31)
    n = 1 << 15
    src, dst = [], []
    for h, k in enumerate([1, 31, 32, 33, 63, 64, 65, 255, 256, 257, 511, 1023, 1024, 4095, 4096, 16385]):
        src += [h] * k
        dst += rng.choice(n, size=k, replace=False).tolist()
    m = 12 * n
    src += rng.integers(0, n, m).tolist()
    dst += (rng.zipf(2.0, m) % n).tolist()
    g = d.from_edges(src, dst, n, d.CSR_SYMMETRIZE | d.CSR_DEDUP)
    with d.Graph(g, opts=opts(hot_cache=32, vertex_order=2, block_threads=block, use_tma=tma)) as dg:
        for s in [0, 7, 15, int(rng.integers(0, n))]:
            run_and_check(g, s, graph=dg)
            run_and_check(g, s, graph=dg, parents=False)


def test_hub_first_auto_and_device_input():
    """Auto mode relabels a skewed graph and keeps a uniform one; a graph
    created from device arrays relabels the same way."""
    torch = pytest.importorskip("torch")
    g = d.gen_rmat(17, 16, seed=22)
    src = int(g.pick_sources(1, seed=22)[0])
    off = torch.from_numpy(g.offsets).cuda()
    col = torch.from_numpy(g.cols).cuda()
    with d.Graph(off, col, n=g.n, e=g.e, opts=opts(vertex_order=0)) as dg:
        run_and_check(g, src, graph=dg)
        lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
        pa = torch.empty(g.n, dtype=torch.int32, device="cuda")
        dg.launch(src, lv, pa)
        dg.sync()
        want = oracle.bfs(g.offsets, g.cols, src)
        assert oracle.compare(want, lv.cpu().numpy())["mismatches"] == 0
        assert oracle.validate_tree(g.offsets, g.cols, src, lv.cpu().numpy(), pa.cpu().numpy()) == 0
    grid, _ = d.gen_grid(300, 0.01, seed=22)
    run_and_check(grid, 0, opts(vertex_order=0))


@pytest.mark.parametrize("order", [0, 1])
def test_direction_optimizing(order):
    """Direction-optimising levels give the oracle's levels, a valid BFS tree
    and E_R; RMAT's large levels do run bottom-up."""
    g = d.gen_rmat(17, 16, seed=31)
    with d.Graph(g, opts=opts(direction=1, vertex_order=order)) as dg:
        for s in g.pick_sources(4, seed=31):
            run_and_check(g, int(s), graph=dg)
        prof = dg.last_levels(64)
        assert any(r["probe"] == 2 for r in prof)          # some level went bottom-up
        assert prof[1]["probe"] != 2 or prof[0]["probe"] != 2  # not every level
    grid, _ = d.gen_grid(200, 0.02, seed=31)
    with d.Graph(grid, opts=opts(direction=1)) as dg:
        run_and_check(grid, 0, graph=dg)
    # a disconnected undirected graph: unreached vertices stay -1
    two = d.from_edges([0, 1, 5, 6], [1, 2, 6, 7], 9, d.CSR_SYMMETRIZE | d.CSR_DEDUP)
    with d.Graph(two, opts=opts(direction=1)) as dg:
        run_and_check(two, 0, graph=dg)


def test_direction_optimizing_needs_undirected():
    directed = d.gen_zipf_geometric(5000, 4.7, 2.1, seed=3)
    with pytest.raises(d.DfqError) as e:
        d.Graph(directed, opts=opts(direction=1))
    assert e.value.name == "EINVAL"
    g = d.gen_rmat(10, 8, seed=3)
    with d.Graph(g) as dg:  # created top-down only: asking for bottom-up later is refused
        o = dg.opts()
        o.direction = 1
        dg.set_opts(o)
        with pytest.raises(d.DfqError):
            dg.bfs(0)


def test_repeated_runs_identical():
    g = d.gen_rmat(15, 16, seed=8)
    src = int(g.pick_sources(1, seed=8)[0])
    with d.Graph(g) as dg:
        first, _, _ = dg.bfs(src)
        first = first.copy()
        for _ in range(20):
            lv, _, _ = dg.bfs(src)
            assert np.array_equal(lv, first)
    assert oracle.compare(oracle.bfs(g.offsets, g.cols, src), first)["mismatches"] == 0


def test_device_buffers_and_launch_api():
    torch = pytest.importorskip("torch")
    g = d.gen_rmat(14, 8, seed=9)
    src = int(g.pick_sources(1, seed=9)[0])
    off = torch.from_numpy(g.offsets).cuda()
    cols = torch.from_numpy(g.cols).cuda()
    with d.Graph(off, cols, n=g.n, e=g.e) as dg:  # device-pointer CSR input
        lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
        pa = torch.empty(g.n, dtype=torch.int32, device="cuda")
        dg.bfs(src, levels_out=lv, parents_out=pa)
        want = oracle.bfs(g.offsets, g.cols, src)
        assert oracle.compare(want, lv.cpu().numpy())["mismatches"] == 0
        assert oracle.validate_tree(g.offsets, g.cols, src, lv.cpu().numpy(), pa.cpu().numpy()) == 0
        lv2 = torch.full((g.n,), 7, dtype=torch.int32, device="cuda")
        dg.launch(src, lv2)
        dg.sync()
        assert torch.equal(lv, lv2)
        st = dg.last_stats()
        assert st.edges == oracle.reached_edges(g.offsets, want)


@pytest.mark.parametrize("order", [1, 2])
def test_pinned_host_outputs(order):
    """Pinned host outputs are written by the kernel's last pass (no separate
    copy): levels and parents equal the pageable-buffer path's, with and
    without hub-first ids, for levels alone, parents alone and both; the
    statistics of a pinned run match too."""
    torch = pytest.importorskip("torch")
    g = d.gen_rmat(15, 16, seed=41)
    with d.Graph(g, opts=opts(vertex_order=order)) as dg:
        for s in g.pick_sources(3, seed=41):
            s = int(s)
            want = oracle.bfs(g.offsets, g.cols, s)
            lv_h = torch.full((g.n,), 5, dtype=torch.int32).pin_memory()
            pa_h = torch.full((g.n,), 5, dtype=torch.int32).pin_memory()
            _, _, st = dg.bfs(s, levels_out=lv_h, parents_out=pa_h)
            assert oracle.compare(want, lv_h.numpy())["mismatches"] == 0
            assert oracle.validate_tree(g.offsets, g.cols, s, lv_h.numpy(), pa_h.numpy()) == 0
            assert st.edges == oracle.reached_edges(g.offsets, want)
            assert st.reached == int((want >= 0).sum())
            # pinned levels with pageable parents, and the other way round
            lv2 = torch.full((g.n,), 5, dtype=torch.int32).pin_memory()
            pa2 = np.full(g.n, 5, np.int32)
            dg.bfs(s, levels_out=lv2, parents_out=pa2)
            assert torch.equal(lv2, lv_h)
            assert oracle.validate_tree(g.offsets, g.cols, s, lv2.numpy(), pa2) == 0
            lv3 = np.full(g.n, 5, np.int32)
            pa3 = torch.full((g.n,), 5, dtype=torch.int32).pin_memory()
            dg.bfs(s, levels_out=lv3, parents_out=pa3)
            assert np.array_equal(lv3, lv_h.numpy())
            assert oracle.validate_tree(g.offsets, g.cols, s, lv3, pa3.numpy()) == 0
            lv4 = torch.full((g.n,), 5, dtype=torch.int32).pin_memory()
            dg.bfs(s, levels_out=lv4)
            assert torch.equal(lv4, lv_h)


@pytest.mark.parametrize("level", [1, 2])
def test_barrier_timeout_reported_and_graph_usable(level):
    """Failure path without a fault: with stall_test_level the last block
    skips one grid-barrier arrival, so every block's bounded wait runs out
    after timeout_ms; the call returns ETIMEOUT (through dfq_bfs and through
    dfq_bfs_launch + sync) and the same graph then runs exact BFS again."""
    import time
    torch = pytest.importorskip("torch")
    g = d.gen_rmat(14, 8, seed=12)
    src = int(g.pick_sources(1, seed=12)[0])
    assert oracle.bfs(g.offsets, g.cols, src).max() >= level  # the stalled barrier is reached
    with d.Graph(g, opts=opts(timeout_ms=20)) as dg:
        dg.set_opts({"stall_test_level": level})
        t0 = time.perf_counter()
        with pytest.raises(d.DfqError) as e:
            dg.bfs(src)
        assert e.value.name == "ETIMEOUT" and "barrier" in str(e.value)
        assert time.perf_counter() - t0 < 5.0
        lv = torch.full((g.n,), 3, dtype=torch.int32, device="cuda")
        dg.launch(src, lv)
        with pytest.raises(d.DfqError) as e:
            dg.sync()
        assert e.value.name == "ETIMEOUT"
        dg.set_opts({"stall_test_level": 0})
        run_and_check(g, src, graph=dg)
        dg.launch(src, lv)
        dg.sync()
        assert oracle.compare(oracle.bfs(g.offsets, g.cols, src), lv.cpu().numpy())["mismatches"] == 0


def test_graphs_needing_different_shared_memory_alternate():
    """The single-source kernel is one function shared by every graph handle
    and by the no-alloc entry point: handles whose layouts need different
    shared memory (a 32 KB hot cache, the smallest pieces) alternate on one
    device, with no-alloc runs in between, and every run stays exact."""
    torch = pytest.importorskip("torch")
    g = d.gen_rmat(14, 16, seed=5)
    src = int(g.pick_sources(1, seed=5)[0])
    want = oracle.bfs(g.offsets, g.cols, src)
    off = torch.from_numpy(g.offsets).cuda()
    cols = torch.from_numpy(g.cols).cuda()
    big = d.Graph(g, opts=opts(hot_cache=32, vertex_order=2))
    small = d.Graph(g, opts=opts(piece_edges=64, large_min_degree=64))
    try:
        for _ in range(2):
            for dg in (big, small):
                run_and_check(g, src, graph=dg)
                lv = torch.full((g.n,), 9, dtype=torch.int32, device="cuda")
                d.bfs_noalloc(off, cols, g.n, g.e, src, lv)
                torch.cuda.synchronize()
                assert oracle.compare(want, lv.cpu().numpy())["mismatches"] == 0
    finally:
        big.close()
        small.close()


def test_invalid_source_and_csr():
    g = d.gen_rmat(8, 4, seed=1)
    with d.Graph(g) as dg:
        with pytest.raises(d.DfqError) as e:
            dg.bfs(g.n)
        assert e.value.name == "EINVAL"
        with pytest.raises(d.DfqError):
            dg.set_opts(opts(block_threads=300))
    bad = d.Csr(g.offsets.copy(), g.cols.copy())
    bad.cols[0] = g.n + 5
    with pytest.raises(d.DfqError) as e:
        d.Graph(bad)
    assert e.value.name == "EFORMAT"
    torch = pytest.importorskip("torch")
    off = torch.from_numpy(g.offsets).cuda()
    cols = torch.from_numpy(bad.cols).cuda()
    with pytest.raises(d.DfqError) as e:
        d.Graph(off, cols, n=g.n, e=g.e)
    assert e.value.name == "EFORMAT"


def test_single_vertex_and_empty_graph():
    g = d.from_edges([], [], 1)
    run_and_check(g, 0)
    g = d.from_edges([], [], 50)
    run_and_check(g, 13)


@pytest.mark.parametrize("kw", [{"l2_persist": 1}, {"blocks_per_sm": 1}, {"blocks_per_sm": 2},
                                {"blocks_per_sm": 1, "block_threads": 1024, "hot_cache": 32},
                                {"l2_persist": 1, "hot_cache": 32, "vertex_order": 2}])
def test_autotuner_axes_keep_parity(kw):
    """Every option the autotuner can pick runs bit-exact: the L2-persisting
    bitmap window, capped blocks per SM, and the hot-vertex cache, on a
    skewed graph (hub-first ids) and a grid."""
    rm = d.gen_rmat(17, 16, seed=41)
    grid, _ = d.gen_grid(256, 0.02, seed=41)
    for g, srcs in [(rm, [int(x) for x in rm.pick_sources(3, seed=41)]), (grid, [0, grid.n // 2])]:
        with d.Graph(g, opts=opts(**kw)) as dg:
            for s in srcs:
                run_and_check(g, s, graph=dg)
                run_and_check(g, s, graph=dg, parents=False)


def test_autotune_keeps_parity():
    g = d.gen_rmat(15, 16, seed=10)
    srcs = g.pick_sources(2, seed=10)
    with d.Graph(g) as dg:
        best = dg.autotune(srcs)
        assert best.block_threads in (256, 512, 1024)
        for s in srcs:
            run_and_check(g, int(s), graph=dg)


def _check_all_sources(g, srcs, parents, opts=None):
    """Every source through dfq_bfs, bit-exact against the oracle (run on the
    host's cores in threads: ctypes releases the GIL), parents validated as a
    BFS tree, kernel E_R and reached count equal to the oracle's."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    oracle.lib()
    workers = min(16, os.cpu_count() or 1)
    with d.Graph(g, opts=opts) as dg, ThreadPoolExecutor(max_workers=workers) as ex:
        wants = [ex.submit(oracle.bfs, g.offsets, g.cols, int(s)) for s in srcs]
        checks = []
        for i, s in enumerate(srcs):
            lv, pa, st = dg.bfs(int(s), parents=parents)

            def check(i=i, s=int(s), lv=lv, pa=pa, st=st):
                want = wants[i].result()
                cmp = oracle.compare(want, lv)
                tree = oracle.validate_tree(g.offsets, g.cols, s, lv, pa) if parents else 0
                er = oracle.reached_edges(g.offsets, want)
                wants[i] = None
                return s, cmp["mismatches"], tree, st.edges == er, st.reached == int((want >= 0).sum())
            checks.append(ex.submit(check))
        bad = [c.result() for c in checks]
    bad = [b for b in bad if b[1] or b[2] or not b[3] or not b[4]]
    assert not bad, f"sources failing (source, level mismatches, tree, E_R ok, reached ok): {bad[:4]}"


def test_full_size_rmat22_every_source():
    """RMAT scale 22, edge factor 16: all 64 benchmark sources (pick_sources(64,
    seed=1)), levels bit-exact, parents a BFS tree."""
    g = d.gen_rmat(22, 16, seed=1)
    _check_all_sources(g, g.pick_sources(64, seed=1), parents=True)


def test_full_size_grid4096_every_source():
    """The 4096^2 grid with 1% of edges deleted (largest component): all 16
    benchmark sources (4 corners, 12 seeded interior vertices)."""
    import bench
    g, orig = d.gen_grid(4096, 0.01, seed=1)
    srcs = bench.grid_sources(orig, 4096)
    assert len(srcs) == 16
    _check_all_sources(g, srcs, parents=False)


def test_autotune_cache_per_gpu_and_graph_class(tmp_path):
    """dfq_autotune_cached: a miss tunes and writes a JSON entry keyed by GPU
    and graph class; a second graph of the same class reuses it without
    timing; a graph of another class gets its own entry; results stay exact."""
    import json
    cache = tmp_path / "tuned.json"
    g = d.gen_rmat(15, 16, seed=12)
    srcs = g.pick_sources(2, seed=12)
    with d.Graph(g) as dg:
        cls = dg.graph_class()
        assert cls.startswith("skewed-" if dg.hub_first else "even-") and "-n2^15-" in cls, cls
        best, hit = dg.autotune_cached(srcs, cache)
        assert not hit
        for s in srcs:
            run_and_check(g, int(s), graph=dg)
    entries = json.loads(cache.read_text())["entries"]
    assert len(entries) == 1 and entries[0]["class"] == cls
    assert entries[0]["opts"]["block_threads"] == best.block_threads
    h = d.gen_rmat(15, 16, seed=13)
    with d.Graph(h) as dh:
        if dh.graph_class() == cls:  # same class: reused without timing
            again, hit = dh.autotune_cached(h.pick_sources(2, seed=13), cache)
            assert hit and again.as_dict() == best.as_dict()
        run_and_check(h, int(h.pick_sources(1, seed=13)[0]), graph=dh)
    grid, _ = d.gen_grid(128, 0.0, seed=1)
    with d.Graph(grid) as dgr:
        assert dgr.graph_class() == "even-n2^14-d2^2"
        _, hit = dgr.autotune_cached([0, grid.n - 1], cache)
        assert not hit
        run_and_check(grid, 0, graph=dgr)
    assert len(json.loads(cache.read_text())["entries"]) == 2
