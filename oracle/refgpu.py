"""Run the reference's own kernel (oracle/_ref/*.cubin) through
oracle/build/librefgpu.so.  Test and benchmark infrastructure only.

available() says whether the cubins and a GPU are present; RefGpu(kind)
loads one kernel: "dfq" = design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu,
"global" = design/global-q/stripe-sa/gun-sep/lower-bound/bfs.cu.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _b

KINDS = {"dfq": (0, "dfq_shared_atomic_oursep_upper"), "global": (1, "global_stripe_gunsep_lower")}


def cubin(kind: str) -> Path:
    return _b.REF_OUT / f"{KINDS[kind][1]}.cubin"


def available(kind: str = "dfq") -> bool:
    return cubin(kind).exists()


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _b.build_refgpu()
        L = C.CDLL(str(path))
        P = C.POINTER(C.c_int32)
        L.refgpu_error.restype = C.c_char_p
        L.refgpu_open.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]
        L.refgpu_load_graph.argtypes = [C.c_void_p, C.c_int32, C.c_int64, P, P]
        L.refgpu_check_bins.argtypes = [C.c_int, C.c_int32, P, P]
        L.refgpu_bfs.argtypes = [C.c_void_p, C.c_int32, P, C.POINTER(C.c_float)]
        L.refgpu_close.argtypes = [C.c_void_p]
        L.refgpu_close.restype = None
        L.refgpu_grid.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class RefGpu:
    def __init__(self, kind: str = "dfq"):
        self.kind = kind
        self.code = KINDS[kind][0]
        h = C.c_void_p()
        if lib().refgpu_open(str(cubin(kind)).encode(), self.code, C.byref(h)) != 0:
            raise RuntimeError(lib().refgpu_error().decode())
        self.h = h
        self.n = 0

    @property
    def grid(self) -> int:
        return lib().refgpu_grid(self.h)

    def load(self, offsets, cols) -> None:
        self.off = np.ascontiguousarray(offsets, np.int32)
        self.cols = np.ascontiguousarray(cols, np.int32)
        self.n = len(self.off) - 1
        z = self.cols if len(self.cols) else np.zeros(1, np.int32)
        if lib().refgpu_load_graph(self.h, self.n, len(self.cols), _p(self.off), _p(z)) != 0:
            raise RuntimeError(lib().refgpu_error().decode())

    def safe_for(self, oracle_levels) -> tuple[bool, str]:
        """Whether the reference kernel's static queues hold every level."""
        lv = np.ascontiguousarray(oracle_levels, np.int32)
        ok = lib().refgpu_check_bins(self.code, self.n, _p(self.off), _p(lv)) == 0
        return ok, ("" if ok else lib().refgpu_error().decode())

    def bfs(self, src: int):
        """(levels int32, '- Time' ms).  Call safe_for() first."""
        lv = np.empty(self.n, np.int32)
        ms = C.c_float()
        if lib().refgpu_bfs(self.h, int(src), _p(lv), C.byref(ms)) != 0:
            raise RuntimeError(lib().refgpu_error().decode())
        return lv, float(ms.value)

    def close(self):
        if self.h:
            lib().refgpu_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
