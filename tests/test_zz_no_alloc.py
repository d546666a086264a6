"""dfq_bfs_noalloc: the entry point for callers that cannot call cudaMalloc
(a framework that owns the GPU's memory through its own pool, a server that
fixes its HBM budget at start-up, code that cannot accept the device-wide
stall of cudaMalloc/cudaFree).  It takes caller-owned device buffers and uses
the library's fixed scratch array instead of allocating.

Checked here through the C ABI against the existing entry point (dfq_bfs on a
dfq_graph): levels must be identical, bit for bit, on two calls in a row
(the scratch array keeps the previous call's contents, so the second call
also checks that nothing stale leaks through), and parents must form a BFS
tree.  This file is collected last so a failure here leaves every other
test already run."""
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


def device_csr(torch, g):
    off = torch.from_numpy(g.offsets).cuda()
    cols = torch.from_numpy(g.cols if g.e else np.zeros(4, np.int32)).cuda()
    return off, cols


def test_noalloc_matches_dfq_bfs_two_calls(torch):
    g = d.gen_rmat(15, 16, seed=77)  # 32768 vertices, ~0.9M edges: well inside the scratch bound
    srcs = [int(s) for s in g.pick_sources(2, seed=77)]
    off, cols = device_csr(torch, g)
    with d.Graph(g) as dg:
        for call, src in enumerate([srcs[0], srcs[1]]):
            want, _, wst = dg.bfs(src)                       # existing entry point
            lv = torch.full((g.n,), 12345, dtype=torch.int32, device="cuda")
            pa = torch.full((g.n,), 12345, dtype=torch.int32, device="cuda")
            st = d.bfs_noalloc(off, cols, g.n, g.e, src, lv, pa)
            got = lv.cpu().numpy()
            assert np.array_equal(got, want), f"call {call}: levels differ from dfq_bfs"
            assert oracle.compare(oracle.bfs(g.offsets, g.cols, src), got)["mismatches"] == 0
            assert oracle.validate_tree(g.offsets, g.cols, src, got, pa.cpu().numpy()) == 0
            assert st.edges == wst.edges and st.reached == wst.reached and st.depth == wst.depth


def test_noalloc_allocates_no_device_memory(torch):
    """What the entry point exists for: after a first call (which sets up the
    device), further calls change neither the device's free memory nor what
    torch's caching allocator holds."""
    g = d.gen_rmat(14, 16, seed=80)
    off, cols = device_csr(torch, g)
    lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
    pa = torch.empty(g.n, dtype=torch.int32, device="cuda")
    srcs = [int(s) for s in g.pick_sources(4, seed=80)]
    d.bfs_noalloc(off, cols, g.n, g.e, srcs[0], lv, pa)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for s in srcs:
        d.bfs_noalloc(off, cols, g.n, g.e, s, lv, pa)
        d.bfs_noalloc(off, cols, g.n, g.e, s, lv)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    assert torch.cuda.memory_reserved() == reserved0
    assert oracle.compare(oracle.bfs(g.offsets, g.cols, srcs[-1]), lv.cpu().numpy())["mismatches"] == 0


def test_noalloc_same_source_twice_without_parents(torch):
    g, _ = d.gen_grid(300, 0.02, seed=78)
    off, cols = device_csr(torch, g)
    with d.Graph(g) as dg:
        want, _, _ = dg.bfs(0)
    for _ in range(2):
        lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
        d.bfs_noalloc(off, cols, g.n, g.e, 0, lv)
        assert np.array_equal(lv.cpu().numpy(), want)
        assert oracle.compare(oracle.bfs(g.offsets, g.cols, 0), lv.cpu().numpy())["mismatches"] == 0


def test_noalloc_rejects_what_it_cannot_hold(torch):
    g = d.gen_rmat(10, 8, seed=79)
    off, cols = device_csr(torch, g)
    lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
    # more vertices than the fixed scratch array can serve: rejected before any launch
    with pytest.raises(d.DfqError) as e:
        d.bfs_noalloc(off, cols, 5_000_000, g.e, 0, lv)
    assert e.value.name == "ENOMEM" and "scratch" in str(e.value)
    # a column array that is not 16-byte aligned is refused (int4 loads need it)
    rc = d.lib().dfq_bfs_noalloc(off.data_ptr(), cols.data_ptr() + 4, g.n, g.e - 1, 0, lv.data_ptr(), None,
                                 None, None)
    assert rc == -1 and b"16-byte aligned" in d.lib().dfq_last_error()
    # a malformed CSR is caught by the device-side check, not by the traversal
    bad_cols = cols.clone()
    bad_cols[3] = g.n + 7
    with pytest.raises(d.DfqError) as e:
        d.bfs_noalloc(off, bad_cols, g.n, g.e, 0, lv)
    assert e.value.name == "EFORMAT"
