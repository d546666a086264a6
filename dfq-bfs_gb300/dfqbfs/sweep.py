"""Design-sweep runner in the layout of the reference's plot.py.

plot.py (plot.py:16-44) runs every program in ``bin/`` on every graph in
``data/`` (both sorted by name) ``cycle`` times as ``<bin>/<B> <data>/<D> 8``,
takes the second-to-last whitespace token of each run's stdout (the
``- Time  = <ms>ms`` line of every DFQ-BFS program, minus its ``ms``), and
writes the mean per (program, graph) to ``result.csv`` and a grouped bar chart
to ``result.png``.  This module does the same without pandas:

* ``result.csv`` has plot.py's layout: tab-separated, a header line
  ``<tab>benchmark<tab><B1><tab><B2>...`` and one row per graph
  ``<row index><tab><D><tab><mean ms of B1>...`` (what ``DataFrame.to_csv(sep='\\t')``
  writes for plot.py's table);
* ``result.png`` is drawn when matplotlib can be imported (plot.py always needs
  it), else skipped with a note.

The reference's design-space tree is one program per variant; here variants
are options of one program, so ``--make-variants DIR`` writes small wrapper
programs into DIR, each running ``bfs`` with one option set (``--opt``), to be
swept side by side with the reference's own rebuilt programs.

Usage::

    python -m dfqbfs.sweep CYCLE [--data data] [--bin bin] [--csv result.csv]
                           [--png result.png] [--arg 8] [--timeout S]
    python -m dfqbfs.sweep --make-variants bin
"""
from __future__ import annotations

import argparse
import os
import shlex
import stat
import subprocess
import sys
from pathlib import Path

# option sets written by --make-variants: name -> bfs --opt arguments
VARIANTS = {
    "dfq_default": [],
    "dfq_claim_at_once": ["probe_first=0"],
    "dfq_probe_always": ["probe_first=1"],
    "dfq_no_tma": ["use_tma=0"],
    "dfq_input_ids": ["vertex_order=1"],
    "dfq_no_hot_cache": ["hot_cache=-1"],
    "dfq_large128": ["large_min_degree=128", "piece_edges=128"],
    "dfq_large1024": ["large_min_degree=1024", "piece_edges=512"],
    "dfq_block1024": ["block_threads=1024"],
}


def parse_time_ms(stdout: str) -> float:
    """plot.py:33: the second-to-last whitespace token, without its 'ms'."""
    toks = stdout.split()
    if len(toks) < 2 or not toks[-2].endswith("ms"):
        raise ValueError(f"no '<time>ms' as the second-to-last token in output ending {stdout[-200:]!r}")
    return float(toks[-2][:-2])


def run_sweep(cycle: int, data_dir: Path, bin_dir: Path, arg: str = "8", timeout: float | None = None,
              log=print) -> tuple[list[str], list[str], list[list[float]]]:
    """Mean time (ms) of every program on every graph: matrix[bin][data]."""
    data = sorted(os.listdir(data_dir))
    bins = sorted(os.listdir(bin_dir))
    matrix = [[0.0] * len(data) for _ in bins]
    for i, b in enumerate(bins):
        for j, dname in enumerate(data):
            log(b, dname)
            total = 0.0
            for _ in range(cycle):
                cmd = [str(Path(bin_dir) / b), str(Path(data_dir) / dname), arg]
                p = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
                if p.returncode != 0:
                    raise RuntimeError(f"{' '.join(map(shlex.quote, cmd))} exited {p.returncode}: {p.stderr[-500:]}")
                total += parse_time_ms(p.stdout)
            matrix[i][j] = total / cycle
    return bins, data, matrix


def write_csv(path: Path, bins: list[str], data: list[str], matrix: list[list[float]]) -> None:
    """plot.py's result.csv (tab-separated, index column first)."""
    lines = ["\t".join(["", "benchmark"] + bins)]
    for j, dname in enumerate(data):
        lines.append("\t".join([str(j), dname] + [repr(float(matrix[i][j])) for i in range(len(bins))]))
    Path(path).write_text("\n".join(lines) + "\n")


def read_csv(path: Path) -> tuple[list[str], list[str], list[list[float]]]:
    rows = [l.split("\t") for l in Path(path).read_text().splitlines() if l]
    bins = rows[0][2:]
    data = [r[1] for r in rows[1:]]
    matrix = [[float(r[2 + i]) for r in rows[1:]] for i in range(len(bins))]
    return bins, data, matrix


def write_png(path: Path, bins: list[str], data: list[str], matrix: list[list[float]]) -> bool:
    """plot.py's grouped bar chart (graphs on the x axis, one bar per program)."""
    try:
        import matplotlib
        matplotlib.use("Agg")
        import matplotlib.pyplot as plt
    except Exception:  # pragma: no cover - depends on the machine
        return False
    fig, ax = plt.subplots(figsize=(15, 15))
    width = 0.9 / max(1, len(bins))
    for i, b in enumerate(bins):
        xs = [j - 0.45 + width * (i + 0.5) for j in range(len(data))]
        ax.bar(xs, matrix[i], width=width, label=b)
    ax.set_xticks(range(len(data)))
    ax.set_xticklabels(data, fontsize=15, rotation=45)
    ax.legend()
    fig.savefig(path)
    plt.close(fig)
    return True


def make_variants(out_dir: Path, bfs: Path | None = None, variants: dict | None = None) -> list[Path]:
    """Write one executable wrapper per option set, each running bfs with it."""
    bfs = Path(bfs) if bfs else Path(__file__).resolve().parent.parent / "bin" / "bfs"
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    made = []
    for name, opts in (variants or VARIANTS).items():
        args = " ".join(f"--opt {shlex.quote(o)}" for o in opts)
        # the wrapper passes the graph and plot.py's extra argument through;
        # bfs reads a numeric second argument as the source unless --ref-compat
        body = f'#!/bin/sh\nexec {shlex.quote(str(bfs))} "$1" --ref-compat {args}\n'
        p = out_dir / name
        p.write_text(body)
        p.chmod(p.stat().st_mode | stat.S_IXUSR | stat.S_IXGRP | stat.S_IXOTH)
        made.append(p)
    return made


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m dfqbfs.sweep", description=__doc__.split("\n\n")[0])
    ap.add_argument("cycle", nargs="?", type=int, help="runs per (program, graph), as plot.py's argv[1]")
    ap.add_argument("--data", default="data")
    ap.add_argument("--bin", default="bin")
    ap.add_argument("--csv", default="result.csv")
    ap.add_argument("--png", default="result.png")
    ap.add_argument("--arg", default="8", help="extra argument after the graph (plot.py passes 8)")
    ap.add_argument("--timeout", type=float, default=None, help="seconds per run")
    ap.add_argument("--make-variants", metavar="DIR", help="write option-set wrappers of bfs into DIR and exit")
    a = ap.parse_args(argv)
    if a.make_variants:
        for p in make_variants(Path(a.make_variants)):
            print(p)
        return 0
    if not a.cycle or a.cycle < 1:
        ap.error("cycle (a positive integer) is required")
    bins, data, matrix = run_sweep(a.cycle, Path(a.data), Path(a.bin), a.arg, a.timeout)
    write_csv(Path(a.csv), bins, data, matrix)
    if not write_png(Path(a.png), bins, data, matrix):
        print("matplotlib not importable: wrote", a.csv, "only", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
