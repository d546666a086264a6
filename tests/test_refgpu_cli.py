"""GPU tests of the two outer boundaries:
  * the reference's own kernel (compiled from its sources) agrees with the
    oracle and with this library's kernel on the same graphs and sources;
  * the drop-in `bfs` program prints the reference's stdout block."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import dfqbfs as d
import oracle
from oracle import refgpu

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
EXE = ROOT / "dfq-bfs_gb300" / "bin" / "bfs"


@pytest.mark.parametrize("kind", ["dfq", "global"])
def test_reference_kernel_matches_oracle_and_ours(kind):
    if not refgpu.available(kind):
        pytest.skip("reference cubin not built (reference sources absent where the build ran)")
    graphs = [d.gen_rmat(14, 16, seed=31), d.gen_grid(96, 0.05, seed=32)[0],
              d.gen_zipf_geometric(262144, 4.7, 2.1, seed=1)]
    with refgpu.RefGpu(kind) as ref:
        for g in graphs:
            ref.load(g.offsets, g.cols)
            srcs = [0] if g.n == 262144 else g.pick_sources(3, seed=33).tolist()
            with d.Graph(g) as dg:
                for s in srcs:
                    want = oracle.bfs(g.offsets, g.cols, s)
                    ok, why = ref.safe_for(want)
                    assert ok, why
                    rl, _ = ref.bfs(s)
                    ours, _, _ = dg.bfs(s)
                    assert oracle.compare(want, rl)["near_errors"] == 0
                    assert np.array_equal(ours, want)
                    assert np.array_equal(ours[want >= 0], rl[want >= 0])


def parse_block(out: str) -> dict:
    clean = re.sub(r"\x1b\[[0-9;]*[A-Za-z]", "", out)
    r = {}
    for key, pat in [("nodes", r"# Nodes : (\d+)"), ("edges", r"# Edges : (\d+)"), ("source", r"Source  : (\d+)"),
                     ("dist", r"- Dist  = (\d+)"), ("error", r"- Error = (\d+)"), ("time", r"- Time  = ([0-9.e+-]+)ms")]:
        m = re.findall(pat, clean)
        r[key] = m
    return r


def test_bfs_program_dat_and_snap(tmp_path):
    g = d.gen_rmat(12, 16, seed=41)
    g.source = int(g.pick_sources(1, seed=41)[0])
    g.save(tmp_path / "g.dat", "dat")
    g.save(tmp_path / "g.txt", "snap")
    want = oracle.bfs(g.offsets, g.cols, g.source)
    r = subprocess.run([str(EXE), str(tmp_path / "g.dat"), "--parents"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    b = parse_block(r.stdout)
    assert b["nodes"] == [str(g.n)] and b["edges"] == [str(g.e)] and b["source"] == [str(g.source)]
    assert b["dist"] == [str(want.max())] and b["error"] == ["0"]
    assert r.stdout.endswith("\x1b[0m")
    # plot.py reads the second-to-last whitespace token minus "ms"
    float(r.stdout.split()[-2][:-2])
    touch = f"({int((want >= 0).sum())} / {g.n})"
    assert touch in r.stdout
    # SNAP input; numeric second argument selects the source; --ref-compat ignores it
    r = subprocess.run([str(EXE), str(tmp_path / "g.txt"), "5"], capture_output=True, text=True)
    assert r.returncode == 0 and parse_block(r.stdout)["source"] == ["5"]
    r = subprocess.run([str(EXE), str(tmp_path / "g.dat"), "8", "--ref-compat"], capture_output=True, text=True)
    assert parse_block(r.stdout)["source"] == [str(g.source)]


def test_bfs_program_frontier_profile(tmp_path):
    """--frontier-profile prints the reference profiler's block (Dim / Siz /
    Rng and one "L: a b c e f" line per level) before the result lines, with
    the counts of dfq_frontier_profile on the same levels; "- Time" stays the
    second-to-last token."""
    g = d.gen_rmat(12, 16, seed=43)
    g.source = int(g.pick_sources(1, seed=43)[0])
    g.save(tmp_path / "g.dat", "dat")
    r = subprocess.run([str(EXE), str(tmp_path / "g.dat"), "--frontier-profile", "--profile-tiles",
                        "8,64,1024,16384", "--profile-grid", "72"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    clean = re.sub(r"\x1b\[[0-9;]*[A-Za-z]", "", r.stdout)
    assert "Dim: 72 1024" in clean and "Siz: 8 64 1024 16384 73728" in clean and "Rng: 8 64 1024 16384 inf" in clean
    rows = [list(map(int, m.groups())) for m in re.finditer(r"^(\d+): (\d+) (\d+) (\d+) (\d+) (\d+)$", clean, re.M)]
    want = oracle.bfs(g.offsets, g.cols, g.source)
    idle, _ = d.frontier_profile(g, want, (8, 64, 1024, 16384), 72 * 1024)
    assert [row[0] for row in rows] == list(range(len(idle)))
    assert np.array_equal(np.array([row[1:] for row in rows], np.int64), idle)
    assert clean.index("Rng:") < clean.index("- Dist")
    float(r.stdout.split()[-2][:-2])


def test_bfs_program_interactive(tmp_path):
    g = d.gen_rmat(11, 8, seed=42)
    g.save(tmp_path / "g.dat", "dat")
    s = g.pick_sources(2, seed=42).tolist()
    stdin = f"n\n{s[0]}\nn\n{g.n + 3}\n{s[1]}\ny\n"
    r = subprocess.run([str(EXE), str(tmp_path / "g.dat"), "$"], input=stdin, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    b = parse_block(r.stdout)
    assert len(b["time"]) == 3 and b["error"] == ["0", "0", "0"]
    assert "Exit? [y/n]" in r.stdout
