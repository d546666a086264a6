"""ctypes binding of libdfq (include/dfq.h) for tests, benchmarks and scripts.

Every call goes through the C ABI of dfq-bfs_gb300/lib/libdfq.so; nothing here
computes a BFS itself.  Importing this module never needs a GPU; calls that
launch kernels fail with DfqError when no CUDA device is present.

The reference's interface for this path is the `bfs` program
(design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:181-317): read a graph,
pick a source, run one cooperative launch, print Dist/Touch/Error/Time.  The
classes below mirror those steps: `load`/generators -> `Csr`, `Graph` (device
copy + workspace), `Graph.bfs(source)` -> levels (+ parents) and `Stats`.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
# DFQ_LIB names another build of the library (the profiling build of _build.py)
LIB_PATH = Path(os.environ["DFQ_LIB"]) if os.environ.get("DFQ_LIB") else PKG / "lib" / "libdfq.so"

DFQ_OK = 0
ERRORS = {
    -1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "ETIMEOUT",
    -5: "EFORMAT", -6: "EIO", -7: "EDEVICE", -8: "EBUSY",
}
CSR_SYMMETRIZE, CSR_DEDUP, CSR_NO_SELF_LOOPS = 1, 2, 4
FMT_AUTO, FMT_SNAP, FMT_DAT, FMT_BIN = 0, 1, 2, 3
_FORMATS = {"auto": FMT_AUTO, "snap": FMT_SNAP, "dat": FMT_DAT, "bin": FMT_BIN}

# every symbol include/dfq.h declares (checked by the CPU test suite)
EXPORTS = [
    "dfq_last_error", "dfq_csr_load", "dfq_csr_save", "dfq_csr_from_edges", "dfq_csr_free",
    "dfq_gen_zipf_geometric", "dfq_gen_rmat", "dfq_gen_grid", "dfq_pick_sources", "dfq_free",
    "dfq_opts_default", "dfq_graph_create", "dfq_graph_destroy", "dfq_graph_get_opts",
    "dfq_graph_set_opts", "dfq_graph_stream", "dfq_graph_num_vertices", "dfq_graph_num_edges",
    "dfq_bfs", "dfq_bfs_launch", "dfq_graph_sync", "dfq_bfs_last_stats", "dfq_autotune",
    "dfq_bfs_noalloc", "dfq_bfs_last_trace",
    "dfq_pool_create", "dfq_pool_destroy", "dfq_pool_num_graphs", "dfq_pool_graph_info", "dfq_pool_bfs",
    "dfq_pool_batch", "dfq_server_create", "dfq_server_submit", "dfq_server_poll", "dfq_server_levels",
    "dfq_server_release", "dfq_server_pending", "dfq_server_destroy", "dfq_server_replay",
    "dfq_set_host_threads", "dfq_host_threads", "dfq_bfs_last_levels", "dfq_frontier_profile",
    "dfq_graph_is_hub_first", "dfq_graph_class", "dfq_autotune_cached",
    "dfq_pool_get_opts", "dfq_pool_set_opts", "dfq_pool_autotune",
]
BATCH_GRAPH = 1


class DfqError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code
        self.name = ERRORS.get(code, str(code))


class _Csr(C.Structure):
    _fields_ = [("n", C.c_int32), ("source", C.c_int32), ("e", C.c_int64),
                ("offsets", C.POINTER(C.c_int32)), ("cols", C.POINTER(C.c_int32))]


class Opts(C.Structure):
    _fields_ = [("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("medium_min_degree", C.c_int32), ("large_min_degree", C.c_int32),
                ("local_queue_cap", C.c_int32), ("local_edge_budget", C.c_int32),
                ("piece_edges", C.c_int32),
                ("probe_first", C.c_int32), ("l2_persist", C.c_int32),
                ("use_tma", C.c_int32), ("timeout_ms", C.c_int32),
                ("wide_min_edges", C.c_int32), ("wide_min_degree", C.c_int32),
                ("hot_cache", C.c_int32), ("vertex_order", C.c_int32), ("profile", C.c_int32),
                ("direction", C.c_int32), ("stall_test_level", C.c_int32),
                ("cluster_blocks", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class Query(C.Structure):
    _fields_ = [("graph", C.c_int32), ("source", C.c_int32), ("levels", C.c_void_p), ("parents", C.c_void_p)]


class QueryResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("wide", C.c_int32), ("depth", C.c_int32), ("levels", C.c_int32),
                ("reached", C.c_int64), ("edges", C.c_int64), ("start_us", C.c_double), ("end_us", C.c_double)]


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("ring_capacity", C.c_int32), ("idle_ms", C.c_int32),
                ("with_parents", C.c_int32), ("narrow_queue_cap", C.c_int32)]


class ServerResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("tag", C.c_int64), ("status", C.c_int32), ("wide", C.c_int32),
                ("depth", C.c_int32), ("retried", C.c_int32), ("reached", C.c_int64), ("edges", C.c_int64),
                ("submit_us", C.c_double), ("done_us", C.c_double), ("device_us", C.c_double)]


class LevelInfo(C.Structure):
    _fields_ = [("start_ns", C.c_int64), ("first_done_ns", C.c_int64), ("last_done_ns", C.c_int64),
                ("frontier", C.c_int32), ("edges", C.c_int32), ("overflow", C.c_int32),
                ("pieces", C.c_int32), ("probe", C.c_int32), ("level", C.c_int32), ("phase_ns", C.c_int32 * 4),
                ("claim_ns", C.c_int32 * 4), ("piece_stats", C.c_int64 * 4)]


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_float), ("depth", C.c_int32), ("levels", C.c_int32),
                ("reached", C.c_int64), ("edges", C.c_int64), ("overflow", C.c_int64),
                ("large", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def lib() -> C.CDLL:
    """Load libdfq.so (built by __graft_entry__.build()); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise FileNotFoundError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
    L = C.CDLL(str(LIB_PATH))
    P32 = C.POINTER(C.c_int32)
    L.dfq_last_error.restype = C.c_char_p
    L.dfq_set_host_threads.argtypes = [C.c_int32]
    L.dfq_host_threads.argtypes = []
    L.dfq_host_threads.restype = C.c_int32
    L.dfq_csr_load.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.POINTER(_Csr)]
    L.dfq_csr_save.argtypes = [C.c_char_p, C.POINTER(_Csr), C.c_int32]
    L.dfq_csr_from_edges.argtypes = [P32, P32, C.c_int64, C.c_int32, C.c_int32, C.POINTER(_Csr)]
    L.dfq_csr_free.argtypes = [C.POINTER(_Csr)]
    L.dfq_csr_free.restype = None
    L.dfq_gen_zipf_geometric.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_uint64, C.POINTER(_Csr)]
    L.dfq_gen_rmat.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                               C.c_int32, C.POINTER(_Csr)]
    L.dfq_gen_grid.argtypes = [C.c_int32, C.c_double, C.c_uint64, C.c_int32, C.POINTER(_Csr),
                               C.POINTER(P32)]
    L.dfq_pick_sources.argtypes = [C.POINTER(_Csr), C.c_int32, C.c_uint64, P32]
    L.dfq_frontier_profile.argtypes = [C.POINTER(_Csr), P32, P32, C.c_int64, C.c_int32,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.dfq_free.argtypes = [C.c_void_p]
    L.dfq_free.restype = None
    L.dfq_opts_default.argtypes = [C.POINTER(Opts)]
    L.dfq_opts_default.restype = None
    L.dfq_graph_create.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.POINTER(Opts),
                                   C.POINTER(C.c_void_p)]
    L.dfq_graph_destroy.argtypes = [C.c_void_p]
    L.dfq_graph_get_opts.argtypes = [C.c_void_p, C.POINTER(Opts)]
    L.dfq_graph_set_opts.argtypes = [C.c_void_p, C.POINTER(Opts)]
    L.dfq_graph_stream.argtypes = [C.c_void_p]
    L.dfq_graph_stream.restype = C.c_void_p
    L.dfq_graph_num_vertices.argtypes = [C.c_void_p]
    L.dfq_graph_num_vertices.restype = C.c_int32
    L.dfq_graph_num_edges.argtypes = [C.c_void_p]
    L.dfq_graph_num_edges.restype = C.c_int64
    L.dfq_bfs.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(Stats)]
    L.dfq_bfs_launch.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.dfq_graph_sync.argtypes = [C.c_void_p]
    L.dfq_bfs_last_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    L.dfq_autotune.argtypes = [C.c_void_p, P32, C.c_int32, C.POINTER(Opts)]
    L.dfq_graph_is_hub_first.argtypes = [C.c_void_p]
    L.dfq_graph_is_hub_first.restype = C.c_int32
    L.dfq_graph_class.argtypes = [C.c_void_p, C.c_char_p, C.c_int32]
    L.dfq_autotune_cached.argtypes = [C.c_void_p, P32, C.c_int32, C.c_char_p, C.POINTER(Opts),
                                      C.POINTER(C.c_int32)]
    L.dfq_pool_get_opts.argtypes = [C.c_void_p, C.POINTER(Opts)]
    L.dfq_pool_set_opts.argtypes = [C.c_void_p, C.POINTER(Opts)]
    L.dfq_pool_create.argtypes = [C.POINTER(_Csr), C.c_int32, C.POINTER(Opts), C.POINTER(C.c_void_p)]
    L.dfq_pool_destroy.argtypes = [C.c_void_p]
    L.dfq_pool_num_graphs.argtypes = [C.c_void_p]
    L.dfq_pool_num_graphs.restype = C.c_int32
    L.dfq_pool_graph_info.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int32)]
    L.dfq_pool_bfs.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(Stats)]
    L.dfq_pool_autotune.argtypes = [C.c_void_p, C.POINTER(Query), C.c_int32, C.POINTER(Opts)]
    L.dfq_pool_batch.argtypes = [C.c_void_p, C.POINTER(Query), C.c_int32, C.c_int32, C.POINTER(QueryResult),
                                 C.POINTER(C.c_float)]
    for name in ("dfq_pool_create", "dfq_pool_destroy", "dfq_pool_graph_info", "dfq_pool_bfs", "dfq_pool_batch"):
        getattr(L, name).restype = C.c_int
    L.dfq_server_create.argtypes = [C.c_void_p, C.POINTER(ServerOpts), C.POINTER(C.c_void_p)]
    L.dfq_server_submit.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.POINTER(C.c_int64)]
    L.dfq_server_poll.argtypes = [C.c_void_p, C.POINTER(ServerResult), C.c_int32, C.POINTER(C.c_int32)]
    L.dfq_server_levels.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    L.dfq_server_release.argtypes = [C.c_void_p, C.c_int64]
    L.dfq_server_pending.argtypes = [C.c_void_p]
    L.dfq_server_pending.restype = C.c_int64
    L.dfq_server_destroy.argtypes = [C.c_void_p]
    L.dfq_server_replay.argtypes = [C.c_void_p, P32, P32, C.POINTER(C.c_double), C.c_int32, P32,
                                    C.POINTER(ServerResult)]
    L.dfq_server_replay.restype = C.c_int
    for name in ("dfq_server_create", "dfq_server_submit", "dfq_server_poll", "dfq_server_levels",
                 "dfq_server_release", "dfq_server_destroy"):
        getattr(L, name).restype = C.c_int
    L.dfq_bfs_last_trace.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int32]
    L.dfq_bfs_last_trace.restype = C.c_int
    L.dfq_bfs_last_levels.argtypes = [C.c_void_p, C.POINTER(LevelInfo), C.c_int32]
    L.dfq_bfs_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.c_int32, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.POINTER(Stats)]
    for name in ("dfq_csr_load", "dfq_csr_save", "dfq_csr_from_edges", "dfq_gen_zipf_geometric",
                 "dfq_gen_rmat", "dfq_gen_grid", "dfq_pick_sources", "dfq_graph_create",
                 "dfq_graph_destroy", "dfq_graph_get_opts", "dfq_graph_set_opts", "dfq_bfs",
                 "dfq_bfs_launch", "dfq_graph_sync", "dfq_bfs_last_stats", "dfq_autotune",
                 "dfq_bfs_noalloc"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != DFQ_OK:
        raise DfqError(rc, lib().dfq_last_error().decode(errors="replace"))


def _p32(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Csr:
    """Host CSR graph: offsets[n+1], cols[e] (numpy int32), source hint."""

    def __init__(self, offsets: np.ndarray, cols: np.ndarray, source: int = 0, meta: dict | None = None):
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int32)
        self.cols = np.ascontiguousarray(cols, dtype=np.int32)
        self.source = int(source)
        self.meta = dict(meta or {})

    @property
    def n(self) -> int:
        return len(self.offsets) - 1

    @property
    def e(self) -> int:
        return len(self.cols)

    def degrees(self) -> np.ndarray:
        return np.diff(self.offsets)

    @classmethod
    def _from_c(cls, c: _Csr, meta: dict | None = None) -> "Csr":
        n, e = c.n, c.e
        off = np.ctypeslib.as_array(c.offsets, shape=(n + 1,)).copy() if n >= 0 else np.zeros(1, np.int32)
        cols = np.ctypeslib.as_array(c.cols, shape=(max(e, 1),))[:e].copy() if c.cols else np.zeros(0, np.int32)
        src = c.source
        lib().dfq_csr_free(C.byref(c))
        return cls(off, cols, src, meta)

    def _as_c(self) -> _Csr:
        c = _Csr()
        c.n, c.e, c.source = self.n, self.e, self.source
        c.offsets = _p32(self.offsets)
        c.cols = _p32(self.cols) if self.e else _p32(np.zeros(1, np.int32))
        return c

    def save(self, path: str | os.PathLike, fmt: str = "snap") -> None:
        c = self._as_c()
        check(lib().dfq_csr_save(str(path).encode(), C.byref(c), _FORMATS[fmt]))

    def pick_sources(self, k: int, seed: int) -> np.ndarray:
        out = np.zeros(k, np.int32)
        c = self._as_c()
        check(lib().dfq_pick_sources(C.byref(c), k, seed, _p32(out)))
        return out


def set_host_threads(threads: int) -> None:
    """Host threads for loaders, the CSR builder and generators (0 = default)."""
    check(lib().dfq_set_host_threads(int(threads)))


def host_threads() -> int:
    return int(lib().dfq_host_threads())


REF_PROFILE_TILES = (16, 128, 1024, 8192)  # TILE_SIZ_A/B/C/E of the reference's frontier profiler


def frontier_profile(g: "Csr", levels, tiles=REF_PROFILE_TILES, threads: int = 304 * 1024,
                     max_levels: int | None = None):
    """Idle lanes and frontier counts per level and bin of the reference's
    binned expansion (dfq_frontier_profile): two int64 arrays of shape
    (levels, 5), bins = degree <= tiles[0..3], then the whole-grid bin.
    threads = the reference launch's gridDim.x * blockDim.x (its
    occupancy-sized grid on GB300 is 304 blocks of 1024)."""
    lv = np.ascontiguousarray(levels, dtype=np.int32)
    if lv.shape != (g.n,):
        raise ValueError("levels must hold one entry per vertex")
    t = np.ascontiguousarray(tiles, dtype=np.int32)
    if t.shape != (4,):
        raise ValueError("tiles must be four sizes")
    m = int(max(int(lv.max(initial=-1)) + 1, 0) if max_levels is None else max_levels)
    idle = np.zeros((max(m, 1), 5), np.int64)
    cnt = np.zeros((max(m, 1), 5), np.int64)
    c = g._as_c()
    k = lib().dfq_frontier_profile(C.byref(c), _p32(lv), _p32(t), int(threads), m,
                                   idle.ctypes.data_as(C.POINTER(C.c_int64)),
                                   cnt.ctypes.data_as(C.POINTER(C.c_int64)))
    if k < 0:
        check(k)
    return idle[:k], cnt[:k]


def load(path: str | os.PathLike, fmt: str = "auto", flags: int = 0) -> Csr:
    c = _Csr()
    check(lib().dfq_csr_load(str(path).encode(), _FORMATS[fmt], flags, C.byref(c)))
    return Csr._from_c(c, {"path": str(path)})


def from_edges(src, dst, n: int, flags: int = 0) -> Csr:
    s = np.ascontiguousarray(src, dtype=np.int32)
    d = np.ascontiguousarray(dst, dtype=np.int32)
    if len(s) != len(d):
        raise ValueError("src and dst lengths differ")
    c = _Csr()
    z = np.zeros(1, np.int32)
    check(lib().dfq_csr_from_edges(_p32(s if len(s) else z), _p32(d if len(d) else z), len(s), n, flags,
                                   C.byref(c)))
    return Csr._from_c(c)


def gen_zipf_geometric(n: int, mean_deg: float = 4.7, alpha: float = 2.1, seed: int = 1) -> Csr:
    c = _Csr()
    check(lib().dfq_gen_zipf_geometric(n, mean_deg, alpha, seed, C.byref(c)))
    return Csr._from_c(c, {"generator": "zipf_geometric", "n": n, "mean_deg": mean_deg, "alpha": alpha,
                           "seed": seed})


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1, flags: int = CSR_SYMMETRIZE | CSR_DEDUP | CSR_NO_SELF_LOOPS) -> Csr:
    cs = _Csr()
    check(lib().dfq_gen_rmat(scale, edge_factor, a, b, c, seed, flags, C.byref(cs)))
    return Csr._from_c(cs, {"generator": "rmat", "scale": scale, "edge_factor": edge_factor,
                            "abc": [a, b, c], "seed": seed, "flags": flags})


def gen_grid(side: int, delete_frac: float = 0.01, seed: int = 1, keep_lcc: bool = True):
    """Returns (Csr, orig_ids) where orig_ids[v] is v's row-major id in the full grid."""
    cs = _Csr()
    ids = C.POINTER(C.c_int32)()
    check(lib().dfq_gen_grid(side, delete_frac, seed, int(keep_lcc), C.byref(cs), C.byref(ids)))
    n = cs.n
    orig = np.ctypeslib.as_array(ids, shape=(max(n, 1),))[:n].copy()
    lib().dfq_free(ids)
    return Csr._from_c(cs, {"generator": "grid", "side": side, "delete_frac": delete_frac, "seed": seed,
                            "keep_lcc": keep_lcc}), orig


def default_opts() -> Opts:
    o = Opts()
    lib().dfq_opts_default(C.byref(o))
    return o


def _ptr(x) -> int:
    """Address of a numpy array or a torch tensor (host or device)."""
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return int(x.data_ptr())


class Graph:
    """Device-resident graph with its BFS workspace (dfq_graph_create)."""

    def __init__(self, csr_or_offsets, cols=None, n: int | None = None, e: int | None = None,
                 opts: Opts | None = None):
        if isinstance(csr_or_offsets, Csr):
            csr = csr_or_offsets
            self._keep = (csr.offsets, csr.cols if csr.e else np.zeros(1, np.int32))
            off_p, col_p, n, e = _ptr(csr.offsets), _ptr(self._keep[1]), csr.n, csr.e
        else:  # device tensors / arrays with explicit sizes
            self._keep = (csr_or_offsets, cols)
            off_p, col_p = _ptr(csr_or_offsets), _ptr(cols)
        h = C.c_void_p()
        check(lib().dfq_graph_create(off_p, col_p, n, e, C.byref(opts) if opts is not None else None,
                                     C.byref(h)))
        self.h = h
        self.n, self.e = n, e

    def close(self) -> None:
        if getattr(self, "h", None):
            check(lib().dfq_graph_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self) -> int:
        return lib().dfq_graph_stream(self.h) or 0

    def opts(self) -> Opts:
        o = Opts()
        check(lib().dfq_graph_get_opts(self.h, C.byref(o)))
        return o

    def set_opts(self, o: Opts | dict) -> None:
        if isinstance(o, dict):
            base = self.opts()
            for k, v in o.items():
                setattr(base, k, v)
            o = base
        check(lib().dfq_graph_set_opts(self.h, C.byref(o)))

    def bfs(self, source: int, parents: bool = False, levels_out=None, parents_out=None):
        """Synchronous BFS.  Returns (levels, parents or None, Stats).  Outputs go
        to the given arrays/tensors (host or device) or to new numpy arrays."""
        lv = levels_out if levels_out is not None else np.empty(self.n, np.int32)
        pa = parents_out if parents_out is not None else (np.empty(self.n, np.int32) if parents else None)
        st = Stats()
        check(lib().dfq_bfs(self.h, int(source), _ptr(lv), _ptr(pa) if pa is not None else None,
                            C.byref(st)))
        return lv, pa, st

    def launch(self, source: int, levels_dev, parents_dev=None) -> None:
        check(lib().dfq_bfs_launch(self.h, int(source), _ptr(levels_dev),
                                   _ptr(parents_dev) if parents_dev is not None else None))

    def sync(self) -> None:
        check(lib().dfq_graph_sync(self.h))

    def last_stats(self) -> Stats:
        st = Stats()
        check(lib().dfq_bfs_last_stats(self.h, C.byref(st)))
        return st

    def last_trace(self, max_levels: int = 64):
        """(start_ns[int64], frontier[int32]) of the first levels of the last launch."""
        ns = np.zeros(max_levels, np.int64)
        fr = np.zeros(max_levels, np.int32)
        k = lib().dfq_bfs_last_trace(self.h, ns.ctypes.data_as(C.POINTER(C.c_int64)), _p32(fr), max_levels)
        if k < 0:
            check(k)
        return ns[:k], fr[:k]

    def last_levels(self, max_levels: int = 64) -> list[dict]:
        """Per-level profile of the last launch: frontier, edges scanned,
        overflow entries, pieces, probe flag, and the level's time split into
        work until the last block finished (us_work), the spread of block
        finish times (us_spread) and the barrier until the next level began
        (us_barrier; absent for the final level)."""
        buf = (LevelInfo * max_levels)()
        k = lib().dfq_bfs_last_levels(self.h, buf, max_levels)
        if k < 0:
            check(k)
        out = []
        for i in range(k):
            r = buf[i]
            row = {"level": r.level, "frontier": r.frontier, "edges": r.edges, "overflow": r.overflow,
                   "pieces": r.pieces, "probe": r.probe}
            if any(r.claim_ns):
                row["us_claim_steps"] = [round(x / 1e3, 2) for x in r.claim_ns]
            if any(r.piece_stats):
                np_ = max(r.piece_stats[0], 1)
                row["pieces_staged"] = r.piece_stats[0]
                row["us_per_piece_wait_expand"] = [round(r.piece_stats[1] / np_ / 1e3, 3),
                                                   round(r.piece_stats[2] / np_ / 1e3, 3)]
                row["ms_claim_drains_all_warps"] = round(r.piece_stats[3] / 1e6, 3)
            if r.last_done_ns:
                row["us_phases"] = [round(x / 1e3, 2) for x in r.phase_ns]
                row["us_work"] = (r.last_done_ns - r.start_ns) / 1e3
                row["us_spread"] = (r.last_done_ns - r.first_done_ns) / 1e3
                if i + 1 < k:
                    row["us_barrier"] = (buf[i + 1].start_ns - r.last_done_ns) / 1e3
            out.append(row)
        return out

    def autotune(self, sources) -> Opts:
        s = np.ascontiguousarray(sources, dtype=np.int32)
        o = Opts()
        check(lib().dfq_autotune(self.h, _p32(s), len(s), C.byref(o)))
        return o

    @property
    def hub_first(self) -> bool:
        return lib().dfq_graph_is_hub_first(self.h) == 1

    def graph_class(self) -> str:
        buf = C.create_string_buffer(128)
        k = lib().dfq_graph_class(self.h, buf, len(buf))
        if k < 0:
            check(k)
        return buf.value.decode()

    def autotune_cached(self, sources, cache_path) -> tuple[Opts, bool]:
        """dfq_autotune_cached: (options installed, True if they came from the cache)."""
        s = np.ascontiguousarray(sources, dtype=np.int32)
        o = Opts()
        hit = C.c_int32()
        check(lib().dfq_autotune_cached(self.h, _p32(s), len(s), str(cache_path).encode(), C.byref(o),
                                        C.byref(hit)))
        return o, bool(hit.value)


NOALLOC_SCRATCH_BYTES = 32 << 20


def bfs_noalloc(offsets_dev, cols_dev, n: int, e: int, source: int, levels_dev, parents_dev=None,
                stream: int = 0) -> Stats:
    """dfq_bfs_noalloc: BFS over caller-owned device buffers with the library's
    fixed scratch array (no allocation).  Returns the Stats (kernel_ms = 0)."""
    st = Stats()
    check(lib().dfq_bfs_noalloc(_ptr(offsets_dev), _ptr(cols_dev), int(n), int(e), int(source),
                                _ptr(levels_dev), _ptr(parents_dev) if parents_dev is not None else None,
                                stream or None, C.byref(st)))
    return st


class Pool:
    """Device-resident pool of graphs (dfq_pool_create) with batched BFS."""

    def __init__(self, graphs: list, opts: Opts | None = None):
        self._keep = graphs
        arr = (_Csr * len(graphs))()
        for i, g in enumerate(graphs):
            arr[i] = g._as_c()
        h = C.c_void_p()
        check(lib().dfq_pool_create(arr, len(graphs), C.byref(opts) if opts is not None else None, C.byref(h)))
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            check(lib().dfq_pool_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self, graph: int):
        n, e, w = C.c_int32(), C.c_int64(), C.c_int32()
        check(lib().dfq_pool_graph_info(self.h, graph, C.byref(n), C.byref(e), C.byref(w)))
        return n.value, e.value, bool(w.value)

    def opts(self) -> Opts:
        o = Opts()
        check(lib().dfq_pool_get_opts(self.h, C.byref(o)))
        return o

    def set_opts(self, o: Opts) -> None:
        check(lib().dfq_pool_set_opts(self.h, C.byref(o)))

    @staticmethod
    def _query_array(queries):
        qa = (Query * len(queries))()
        for i, q in enumerate(queries):
            qa[i].graph, qa[i].source = int(q[0]), int(q[1])
            qa[i].levels = _ptr(q[2])
            qa[i].parents = _ptr(q[3]) if len(q) > 3 and q[3] is not None else None
        return qa

    def autotune(self, queries) -> Opts:
        """dfq_pool_autotune on these queries (same form as batch()); installs
        and returns the winning options."""
        qa = self._query_array(queries)
        o = Opts()
        check(lib().dfq_pool_autotune(self.h, qa, len(queries), C.byref(o)))
        return o

    def bfs(self, graph: int, source: int, levels_dev, parents_dev=None) -> Stats:
        st = Stats()
        check(lib().dfq_pool_bfs(self.h, graph, source, _ptr(levels_dev),
                                 _ptr(parents_dev) if parents_dev is not None else None, C.byref(st)))
        return st

    def batch(self, queries, flags: int = 0, check_status: bool = True):
        """queries: list of (graph, source, levels_dev[, parents_dev]).
        Returns (list of QueryResult, total device ms)."""
        qa = self._query_array(queries)
        res = (QueryResult * len(queries))()
        ms = C.c_float()
        rc = lib().dfq_pool_batch(self.h, qa, len(queries), flags, res, C.byref(ms))
        if check_status:
            check(rc)
        return list(res), ms.value


class Server:
    """Continuous-batching BFS server over a Pool (dfq_server_*)."""

    def __init__(self, pool: Pool, hbm_budget_bytes: int = 0, ring_capacity: int = 0, idle_ms: int = 0,
                 with_parents: bool = False, narrow_queue_cap: int = 0):
        self.pool = pool
        o = ServerOpts(hbm_budget_bytes, ring_capacity, idle_ms, int(with_parents), narrow_queue_cap)
        h = C.c_void_p()
        check(lib().dfq_server_create(pool.h, C.byref(o), C.byref(h)))
        self.h = h
        self._buf = (ServerResult * 4096)()

    def close(self) -> None:
        if getattr(self, "h", None):
            check(lib().dfq_server_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, graph: int, source: int, tag: int = 0) -> int:
        rid = C.c_int64()
        check(lib().dfq_server_submit(self.h, graph, source, tag, C.byref(rid)))
        return rid.value

    def poll(self) -> list:
        cnt = C.c_int32()
        check(lib().dfq_server_poll(self.h, self._buf, len(self._buf), C.byref(cnt)))
        return [ServerResult.from_buffer_copy(self._buf[i]) for i in range(cnt.value)]

    @property
    def pending(self) -> int:
        return lib().dfq_server_pending(self.h)

    def levels(self, rid: int, n: int, parents: bool = False):
        lv = np.empty(n, np.int32)
        pa = np.empty(n, np.int32) if parents else None
        check(lib().dfq_server_levels(self.h, rid, lv.ctypes.data, pa.ctypes.data if pa is not None else None))
        return lv, pa

    def release(self, rid: int) -> None:
        check(lib().dfq_server_release(self.h, rid))

    def replay(self, graphs, sources, arrival_us, keep=None) -> list:
        """dfq_server_replay: submit request i at arrival_us[i]; returns results in request order."""
        g = np.ascontiguousarray(graphs, np.int32)
        s = np.ascontiguousarray(sources, np.int32)
        a = np.ascontiguousarray(arrival_us, np.float64)
        k = np.ascontiguousarray(keep, np.int32) if keep is not None else None
        res = (ServerResult * len(g))()
        check(lib().dfq_server_replay(self.h, _p32(g), _p32(s), a.ctypes.data_as(C.POINTER(C.c_double)), len(g),
                                      _p32(k) if k is not None else None, res))
        return list(res)

    def drain(self, timeout_s: float = 60.0) -> list:
        import time as _t
        out, t0 = [], _t.time()
        while self.pending > 0:
            out += self.poll()
            if _t.time() - t0 > timeout_s:
                raise TimeoutError(f"{self.pending} requests still pending")
        return out + self.poll()
