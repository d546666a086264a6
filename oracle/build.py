"""Build recipe for the oracle (test infrastructure only).

  build_oracle()  gcc oracle.c gen.c -> oracle/build/liboracle.so   (any machine)
  build_refgpu()  g++ refgpu.cpp -> oracle/build/librefgpu.so  (loader of the
                  reference's kernel; driver API, any machine with CUDA)
  build_ref()     compiles the REFERENCE's own kernel sources, where they lie
                  under /root/reference (or $DFQ_REFERENCE), into device code only
                  (oracle/_ref/*.cubin, sm_103a).  Device code carries no host
                  architecture, so a cubin built here runs from the loader
                  built on the GPU machine.  The reference sources need one
                  CUDA 13 shim: cudaMemPrefetchAsync(ptr, n, int device, stream)
                  was removed in CUDA 13 and its host main() calls it
                  (bfs.cu:273-277), so cuda13_compat.h is force-included.
                  Nothing from the reference is copied into this repository.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "build"
REF_OUT = HERE / "_ref"
# where the reference project lies (only the recipe that compiles its kernels
# reads it); DFQ_REFERENCE overrides the default location
REFERENCE = Path(os.environ.get("DFQ_REFERENCE", "/root/reference"))
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CUDA_HOME = str(Path(NVCC).resolve().parent.parent)

# reference kernels built for the GPU baseline (path within the reference project)
REF_KERNELS = {
    # canonical DFQ: shared-memory bins, atomic status-array scan, our-sep, upper-bound
    "dfq_shared_atomic_oursep_upper": "design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu",
    # global-queue baseline: stripe scan, gun-sep bins, lower-bound tiles
    "global_stripe_gunsep_lower": "design/global-q/stripe-sa/gun-sep/lower-bound/bfs.cu",
}


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).exists() and Path(d).stat().st_mtime > t for d in deps)


def _run(cmd) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def build_oracle() -> Path:
    OUT.mkdir(exist_ok=True)
    lib = OUT / "liboracle.so"
    srcs = [HERE / "oracle.c", HERE / "gen.c"]
    if _stale(lib, srcs):
        _run(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", *map(str, srcs), "-o", str(lib), "-lpthread", "-lm"])
    return lib


def build_refgpu() -> Path | None:
    OUT.mkdir(exist_ok=True)
    lib = OUT / "librefgpu.so"
    src = HERE / "refgpu.cpp"
    if not src.exists():
        return None
    if _stale(lib, [src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", str(src), f"-I{CUDA_HOME}/include",
              "-o", str(lib), f"-L{CUDA_HOME}/lib64/stubs", f"-L{CUDA_HOME}/lib64", "-lcuda"])
    return lib


def build_ref() -> dict:
    """Cubins of the reference kernels; only where the reference is present."""
    if not REFERENCE.exists():
        return {}
    REF_OUT.mkdir(exist_ok=True)
    shim = REF_OUT / "cuda13_compat.h"
    shim_text = (
        "#pragma once\n#include <cuda_runtime.h>\n"
        "static inline cudaError_t cudaMemPrefetchAsync(const void* p, size_t n, int dev, cudaStream_t s) {\n"
        "    cudaMemLocation loc; loc.type = cudaMemLocationTypeDevice; loc.id = dev;\n"
        "    return cudaMemPrefetchAsync(p, n, loc, 0u, s);\n}\n")
    if not shim.exists() or shim.read_text() != shim_text:
        shim.write_text(shim_text)
    out = {}
    for name, rel in REF_KERNELS.items():
        src = REFERENCE / rel
        cubin = REF_OUT / f"{name}.cubin"
        if _stale(cubin, [src, shim]):
            _run([NVCC, "-cubin", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-include", str(shim),
                  str(src), "-o", str(cubin)])
        out[name] = str(cubin)
    return out


def build_all() -> dict:
    res = {"oracle": str(build_oracle())}
    rg = build_refgpu()
    if rg:
        res["refgpu"] = str(rg)
    res.update(build_ref())
    return res


if __name__ == "__main__":
    print(build_all())
