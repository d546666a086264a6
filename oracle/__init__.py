"""CPU oracle for DFQ-BFS parity tests.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker; the product (dfq-bfs_gb300/) never imports
it.  Contents:

  * oracle.c (built to oracle/build/liboracle.so): the reference's serial CPU
    BFS (design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:216-253), its
    validation rule (:290-296), BFS-tree validation and E_R.
  * gen.c (same library): the seeded R-MAT generator and source picker,
    restated so the reference-side benchmark arm builds its workload without
    loading the product library (checked byte for byte against it).
  * py_bfs / py_compare: the same algorithm in pure Python, for tiny graphs,
    used to cross-check the C restatement.
  * refgpu: runs the reference's own kernel (compiled from the reference
    sources into oracle/_ref/ by oracle/build.py) on a GPU, to pin the
    restatement against the reference itself.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "build" / "liboracle.so"
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from . import build as _b
            _b.build_oracle()
        L = C.CDLL(str(LIB_PATH))
        P = C.POINTER(C.c_int32)
        L.oracle_bfs.argtypes = [C.c_int32, P, P, C.c_int32, P]
        L.oracle_bfs.restype = C.c_int64
        L.oracle_compare.argtypes = [C.c_int32, P, P, C.POINTER(C.c_int64)]
        L.oracle_compare.restype = C.c_int64
        L.oracle_validate_tree.argtypes = [C.c_int32, P, P, C.c_int32, P, P]
        L.oracle_validate_tree.restype = C.c_int64
        L.oracle_reached_edges.argtypes = [C.c_int32, P, P]
        L.oracle_reached_edges.restype = C.c_int64
        L.oracle_level_histogram.argtypes = [C.c_int32, P, C.POINTER(C.c_int64), C.c_int32]
        L.oracle_level_histogram.restype = C.c_int32
        PP = C.POINTER(P)
        L.gen_rmat_undirected.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                          C.c_int, PP, PP]
        L.gen_rmat_undirected.restype = C.c_int64
        L.gen_pick_sources.argtypes = [C.c_int32, P, C.c_int32, C.c_uint64, P]
        L.gen_pick_sources.restype = C.c_int
        L.gen_free.argtypes = [C.c_void_p]
        L.gen_free.restype = None
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def bfs(offsets, cols, src: int) -> np.ndarray:
    """Levels from the serial oracle (int32, -1 unreached)."""
    off, col = _i32(offsets), _i32(cols)
    n = len(off) - 1
    lv = np.empty(n, np.int32)
    r = lib().oracle_bfs(n, _p(off), _p(col if len(col) else np.zeros(1, np.int32)), int(src), _p(lv))
    if r < 0:
        raise ValueError("oracle_bfs: bad input")
    return lv


def compare(want, got) -> dict:
    """The reference's validation (near_nodes, near_errors, dist) plus extra
    vertices reached only by `got`.  mismatches == 0 means bit-exact."""
    w, g = _i32(want), _i32(got)
    out = (C.c_int64 * 4)()
    m = lib().oracle_compare(len(w), _p(w), _p(g), out)
    return {"near_nodes": out[0], "near_errors": out[1], "dist": out[2], "extra": out[3], "mismatches": m}


def validate_tree(offsets, cols, src: int, levels, parents) -> int:
    """0 if parents form a BFS tree of levels, else 1 + first bad vertex."""
    off, col = _i32(offsets), _i32(cols)
    return int(lib().oracle_validate_tree(len(off) - 1, _p(off), _p(col if len(col) else np.zeros(1, np.int32)),
                                          int(src), _p(_i32(levels)), _p(_i32(parents))))


def reached_edges(offsets, levels) -> int:
    off = _i32(offsets)
    return int(lib().oracle_reached_edges(len(off) - 1, _p(off), _p(_i32(levels))))


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1, threads: int | None = None):
    """(offsets, cols) of the symmetrised, de-duplicated, self-loop-free R-MAT
    graph the product's generator makes with the same arguments."""
    import os
    P = C.POINTER(C.c_int32)
    off_p, col_p = P(), P()
    t = threads if threads is not None else (os.cpu_count() or 1)
    e = lib().gen_rmat_undirected(scale, edge_factor, a, b, c, seed, t, C.byref(off_p), C.byref(col_p))
    if e < 0:
        raise ValueError("gen_rmat_undirected failed")
    n = 1 << scale
    off = np.ctypeslib.as_array(off_p, shape=(n + 1,)).copy()
    cols = np.ctypeslib.as_array(col_p, shape=(max(int(e), 1),))[: int(e)].copy()
    lib().gen_free(C.cast(off_p, C.c_void_p))
    lib().gen_free(C.cast(col_p, C.c_void_p))
    return off, cols


def pick_sources(offsets, k: int, seed: int) -> np.ndarray:
    """k seeded sources among the vertices of out-degree > 0 (the product's
    picker, restated)."""
    off = _i32(offsets)
    out = np.zeros(k, np.int32)
    if lib().gen_pick_sources(len(off) - 1, _p(off), k, seed, _p(out) if k else None) != 0:
        raise ValueError("gen_pick_sources: no vertex with out-degree > 0")
    return out


# ------------------------------------------------------------ pure Python
def py_bfs(offsets, cols, src: int) -> list[int]:
    """bfs.cu:216-253 line by line, for graphs small enough for Python loops."""
    n = len(offsets) - 1
    X = [False] * n
    C_ = [0] * n
    X[src] = True
    F = [src]
    while F:
        F_next = []
        for i in range(len(F) - 1, -1, -1):
            id_ = F[i]
            for j in range(offsets[id_], offsets[id_ + 1]):
                nid = cols[j]
                if not X[nid]:
                    X[nid] = True
                    C_[nid] = C_[id_] + 1
                    F_next.append(nid)
        F = F_next
    return [C_[i] if X[i] else -1 for i in range(n)]
