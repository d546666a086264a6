"""Generate the golden level fixtures from the reference's own kernel.

The reference repository holds no test vectors and its datasets are missing,
so golden levels are produced by running the reference's kernel itself
(compiled from its sources into oracle/_ref/ by oracle/build.py, launched the
way its host code launches it, oracle/refgpu.cpp) on small seeded graphs.
Needs a GPU.  Writes tests/golden/ref_<name>.npz with the graph (offsets,
cols), the sources, the reference levels per source, and the reference
kernel's '- Error' count against the oracle (must be 0 to be kept).

    python tests/golden/make_golden.py [outdir]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT / "dfq-bfs_gb300"), str(ROOT)]

import dfqbfs as d  # noqa: E402
import oracle  # noqa: E402
from oracle import refgpu  # noqa: E402


def graphs():
    out = {}
    out["zipf_geo_4k"] = (d.gen_zipf_geometric(4096, 4.7, 2.1, seed=21), None)
    out["rmat10_ef16"] = (d.gen_rmat(10, 16, seed=22), None)
    out["rmat12_ef8"] = (d.gen_rmat(12, 8, seed=23), None)
    g, _ = d.gen_grid(48, 0.05, seed=24)
    out["grid48_del5"] = (g, None)
    # bin boundaries of the reference kernel (8/9, 64/65, 1024/1025) and of ours
    rng = np.random.default_rng(25)
    n = 6000
    degs = [8, 9, 31, 32, 33, 64, 65, 1023, 1024, 1025, 2047, 2048, 2049]
    src, dst = [], []
    for i, k in enumerate(degs):
        u = i
        for v in rng.choice(n, size=k, replace=False):
            src.append(u); dst.append(int(v))
    m = 20000
    src += rng.integers(0, n, m).tolist(); dst += rng.integers(0, n, m).tolist()
    src += list(range(len(degs))); dst += list(range(1, len(degs) + 1))
    out["bin_boundaries"] = (d.from_edges(src, dst, n, d.CSR_DEDUP), [0])
    out["path_200"] = (d.from_edges(list(range(199)), list(range(1, 200)), 200), [0, 57])
    return out


def main(outdir: Path) -> int:
    outdir.mkdir(parents=True, exist_ok=True)
    if not refgpu.available("dfq"):
        print("reference cubin missing (oracle/_ref); build it where the reference sources are present")
        return 1
    summary = {}
    with refgpu.RefGpu("dfq") as ref:
        for name, (g, srcs) in graphs().items():
            if srcs is None:
                srcs = g.pick_sources(4, seed=5).tolist()
            ref.load(g.offsets, g.cols)
            levels, errors = [], []
            for s in srcs:
                want = oracle.bfs(g.offsets, g.cols, s)
                ok, why = ref.safe_for(want)
                if not ok:
                    raise SystemExit(f"{name}: {why}")
                lv, ms = ref.bfs(s)
                cmp = oracle.compare(want, lv)
                levels.append(lv)
                errors.append(int(cmp["near_errors"]))
            summary[name] = {"n": g.n, "e": g.e, "sources": srcs, "reference_errors": errors}
            if any(errors):
                print(f"{name}: reference kernel disagrees with the oracle: {errors}; not kept")
                continue
            np.savez_compressed(outdir / f"ref_{name}.npz", offsets=g.offsets, cols=g.cols,
                                sources=np.array(srcs, np.int32), levels=np.stack(levels).astype(np.int32),
                                reference_errors=np.array(errors, np.int32))
    (outdir / "golden_summary.json").write_text(json.dumps(summary, indent=1))
    print(json.dumps(summary))
    return 0


if __name__ == "__main__":
    sys.exit(main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent))
