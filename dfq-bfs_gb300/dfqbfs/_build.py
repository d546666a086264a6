"""Build libdfq.so and the drop-in `bfs` program for sm_103a.

Plain nvcc/g++ invocations run in parallel (no make/cmake needed), each
skipped when its output is newer than its inputs.  Outputs stay in the
package tree: lib/libdfq.so, bin/bfs, build/*.o.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent          # dfq-bfs_gb300/
REPO = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = REPO / "include"
BUILD = PKG / "build"
LIB = PKG / "lib"
BIN = PKG / "bin"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CUDA_HOME = str(Path(NVCC).resolve().parent.parent)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                  "--expt-relaxed-constexpr", "-Xptxas", "-O3"]

HOST_SRCS = ["host_graph.cpp", "host_gen.cpp", "autotune.cpp", "host_profile.cpp"]
CUDA_SRCS = ["dfq_api.cu", "dfq_noalloc.cu", "dfq_batch.cu", "dfq_serve.cu", "dfq_cluster.cu"]
HEADERS = ["common.hpp", "dfq_kernel.cuh", "dfq_pool.cuh"]


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, ptxas_info: bool = False, probes: bool = False) -> dict:
    """Compile everything; returns paths of the products.  probes=True makes
    the profiling build instead (claim-step probes compiled in, -DDFQ_CLAIM_PROBES=1)
    into build_probes/ and lib_probes/; load it with DFQ_LIB=<its libdfq.so>."""
    build_dir, lib_dir, bin_dir, nvflags = BUILD, LIB, BIN, NVFLAGS
    if probes:
        build_dir, lib_dir, bin_dir = PKG / "build_probes", PKG / "lib_probes", PKG / "bin_probes"
        nvflags = NVFLAGS + ["-DDFQ_CLAIM_PROBES=1"]
    build_dir.mkdir(exist_ok=True)
    lib_dir.mkdir(exist_ok=True)
    bin_dir.mkdir(exist_ok=True)
    hdeps = [INCLUDE / "dfq.h"] + [CSRC / h for h in HEADERS]
    jobs = []
    objs = []
    for s in HOST_SRCS:
        src, obj = CSRC / s, build_dir / (s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdeps):
            jobs.append(["g++", *CXXFLAGS, f"-I{INCLUDE}", f"-I{CUDA_HOME}/include", "-c", str(src), "-o", str(obj)])
    for s in CUDA_SRCS:
        src, obj = CSRC / s, build_dir / (s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdeps) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([NVCC, *nvflags, *extra, f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)])
    main_src, main_obj = CSRC / "bfs_main.cpp", build_dir / "bfs_main.cpp.o"
    if _stale(main_obj, [main_src] + hdeps):
        jobs.append(["g++", *CXXFLAGS, f"-I{INCLUDE}", "-c", str(main_src), "-o", str(main_obj)])
    logs = []
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd))
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if r.returncode != 0:
            raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if r.stderr.strip():
            logs.append(r.stderr)
    lib = lib_dir / "libdfq.so"
    if _stale(lib, objs):
        _run([NVCC, *ARCH, "-shared", "-cudart", "shared", *map(str, objs), "-o", str(lib), "-lpthread"])
    exe = bin_dir / "bfs"
    if _stale(exe, [main_obj, lib]):
        _run(["g++", str(main_obj), "-o", str(exe), f"-L{lib_dir}", "-ldfq", f"-Wl,-rpath,$ORIGIN/../lib",
              f"-L{CUDA_HOME}/lib64", f"-Wl,-rpath,{CUDA_HOME}/lib64", "-lcudart", "-lpthread"])
    if verbose and logs:
        print("\n".join(logs))
    return {"lib": str(lib), "bin": str(exe), "log": "\n".join(logs)}


if __name__ == "__main__":
    import sys
    out = build(verbose=True, ptxas_info="--ptxas" in sys.argv, probes="--probes" in sys.argv)
    print(out["log"])
    print(out["lib"], out["bin"])
