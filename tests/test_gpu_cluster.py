"""GPU parity of the cluster form of the single-source kernel
(cluster_blocks = C: one thread-block cluster of C blocks runs the BFS, its
levels ending on a cluster barrier in distributed shared memory) against the
CPU oracle, bit for bit, over the same bins and queues as the whole-grid
kernel; its bounded barrier wait on the failure path; and the option's
checks."""
import numpy as np
import pytest

import dfqbfs as d
import oracle
from test_gpu_parity import BOUNDARY_DEGS, opts, run_and_check

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid512():
    return d.gen_grid(512, 0.01, seed=5)[0]


@pytest.fixture(scope="module")
def mixed():
    """Degrees on every bin boundary chained into one component, plus random
    edges: small, medium and large lists, pieces and overflow at one level."""
    rng = np.random.default_rng(7)
    n = 40000
    src, dst = [], []
    for i, k in enumerate(BOUNDARY_DEGS):
        src += [i] * k
        dst += rng.choice(n, size=k, replace=False).tolist()
    src += list(range(len(BOUNDARY_DEGS) - 1))
    dst += list(range(1, len(BOUNDARY_DEGS)))
    src += rng.integers(0, n, 60000).tolist()
    dst += rng.integers(0, n, 60000).tolist()
    return d.from_edges(src, dst, n, d.CSR_DEDUP)


@pytest.mark.parametrize("C", [2, 8, 16])
@pytest.mark.parametrize("B", [512, 1024])
def test_grid(grid512, C, B):
    _, st = run_and_check(grid512, 0, opts(cluster_blocks=C, block_threads=B))
    assert st.depth > 1000


@pytest.mark.parametrize("C", [2, 16])
@pytest.mark.parametrize("tma", [0, 1])
@pytest.mark.parametrize("probe", [0, 1, 2])
def test_bins_and_pieces(mixed, C, tma, probe):
    _, st = run_and_check(mixed, 0, opts(cluster_blocks=C, block_threads=512, use_tma=tma, probe_first=probe,
                                         large_min_degree=256, piece_edges=64))
    assert st.large > 0


@pytest.mark.parametrize("cap", [1, 16])
def test_forced_overflow(cap):
    g = d.gen_rmat(14, 16, seed=3)
    src = int(g.pick_sources(1, seed=3)[0])
    _, st = run_and_check(g, src, opts(cluster_blocks=8, block_threads=1024, local_queue_cap=cap))
    assert st.overflow > 0


def test_hub_first_graph_several_sources():
    """A skewed graph stored hub-first (results mapped back to input ids)."""
    g = d.gen_rmat(17, 16, seed=9)
    with d.Graph(g, opts=opts(cluster_blocks=16, block_threads=512)) as dg:
        assert dg.hub_first
        for s in g.pick_sources(3, seed=9):
            run_and_check(g, int(s), graph=dg)


def test_direction_optimizing_in_a_cluster():
    g = d.gen_rmat(15, 16, seed=2)
    o = opts(direction=1, cluster_blocks=8, block_threads=1024)
    with d.Graph(g, opts=o) as dg:
        src = int(g.pick_sources(1, seed=2)[0])
        lv, pa, _ = dg.bfs(src, parents=True)
    want = oracle.bfs(g.offsets, g.cols, src)
    assert oracle.compare(want, lv)["mismatches"] == 0
    assert oracle.validate_tree(g.offsets, g.cols, src, lv, pa) == 0


def test_alternating_with_the_whole_grid(grid512):
    """The same graph handle switches between the cluster and the whole-grid
    launch; each run is exact."""
    with d.Graph(grid512) as dg:
        for c in (16, 0, 8, 0):
            dg.set_opts({"cluster_blocks": c})
            run_and_check(grid512, 7, graph=dg)


@pytest.mark.parametrize("level", [1, 3])
def test_barrier_timeout_reported_and_graph_usable(level):
    """With stall_test_level the cluster's last block sends no tallies and no
    arrival at one level end: every block's bounded mbarrier wait runs out
    after timeout_ms, all blocks leave together, the call returns ETIMEOUT and
    the same graph then runs exact BFS again."""
    import time
    g = d.gen_rmat(14, 8, seed=12)
    src = int(g.pick_sources(1, seed=12)[0])
    assert oracle.bfs(g.offsets, g.cols, src).max() >= level
    with d.Graph(g, opts=opts(timeout_ms=20, cluster_blocks=8, block_threads=512)) as dg:
        dg.set_opts({"stall_test_level": level})
        t0 = time.perf_counter()
        with pytest.raises(d.DfqError) as e:
            dg.bfs(src)
        assert e.value.name == "ETIMEOUT" and "barrier" in str(e.value)
        assert time.perf_counter() - t0 < 5.0
        dg.set_opts({"stall_test_level": 0})
        run_and_check(g, src, graph=dg)


def test_option_checks(grid512):
    with d.Graph(grid512) as dg:
        with pytest.raises(d.DfqError) as e:
            dg.set_opts({"cluster_blocks": 3})
        assert e.value.name == "EINVAL"
        dg.set_opts({"cluster_blocks": 8, "block_threads": 256})
        with pytest.raises(d.DfqError) as e:
            dg.bfs(0)
        assert e.value.name == "EINVAL" and "cluster" in str(e.value)
        dg.set_opts({"cluster_blocks": 8, "block_threads": 512})
        run_and_check(grid512, 0, graph=dg)


def test_full_size_grid4096_every_source():
    """The 4096^2 grid (1 % of edges deleted, largest component) on one
    cluster of 16 blocks: all 16 benchmark sources."""
    import bench
    from test_gpu_parity import _check_all_sources
    g, orig = d.gen_grid(4096, 0.01, seed=1)
    srcs = bench.grid_sources(orig, 4096)
    _check_all_sources(g, srcs, parents=False, opts=opts(cluster_blocks=16, block_threads=1024))
