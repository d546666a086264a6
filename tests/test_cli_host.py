"""Host logic on the CPU.  The bfs program is built against a test double of
the device entry points (tests/cli_double), whose BFS is a serial queue BFS,
and its output is checked against the oracle - input formats, source
selection, the reference's stdout block, the '$' loop, --json and
--frontier-profile; the GPU tests run the real program.  The host hub-first
renumbering that pools use is checked by a C++ harness built against the
library's host sources."""
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import dfqbfs as d
import oracle

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "dfq-bfs_gb300" / "csrc"


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("cli") / "bfs_host"
    srcs = [CSRC / "bfs_main.cpp", CSRC / "host_graph.cpp", CSRC / "host_profile.cpp",
            ROOT / "tests" / "cli_double" / "dfq_device_double.cpp"]
    subprocess.run([cxx, "-O1", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{CSRC}", *map(str, srcs), "-o", str(out),
                    "-pthread"], check=True)
    return out


def clean(s: str) -> str:
    return re.sub(r"\x1b\[[0-9;]*[A-Za-z]", "", s)


def field(text, pat):
    return re.findall(pat, clean(text))


def test_dat_block_parents_and_time_token(exe, tmp_path):
    g = d.gen_rmat(11, 8, seed=51)
    g.source = int(g.pick_sources(1, seed=51)[0])
    g.save(tmp_path / "g.dat", "dat")
    want = oracle.bfs(g.offsets, g.cols, g.source)
    r = subprocess.run([str(exe), str(tmp_path / "g.dat"), "--parents"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert field(r.stdout, r"# Nodes : (\d+)") == [str(g.n)] and field(r.stdout, r"# Edges : (\d+)") == [str(g.e)]
    assert field(r.stdout, r"Source  : (\d+)") == [str(g.source)]
    assert field(r.stdout, r"- Dist  = (\d+)") == [str(want.max())]
    assert field(r.stdout, r"- Error = (\d+)") == ["0"]
    assert f"({int((want >= 0).sum())} / {g.n})" in r.stdout
    assert r.stdout.endswith("\x1b[0m") and r.stdout.split()[-2] == "0.125ms"


def test_snap_source_argument_ref_compat_and_json(exe, tmp_path):
    g = d.gen_rmat(10, 8, seed=52)
    g.source = 3
    g.save(tmp_path / "g.txt", "snap")
    g.save(tmp_path / "g.dat", "dat")
    r = subprocess.run([str(exe), str(tmp_path / "g.txt"), "7"], capture_output=True, text=True)
    assert r.returncode == 0 and field(r.stdout, r"Source  : (\d+)") == ["7"]
    r = subprocess.run([str(exe), str(tmp_path / "g.dat"), "8", "--ref-compat"], capture_output=True, text=True)
    assert field(r.stdout, r"Source  : (\d+)") == ["3"]
    r = subprocess.run([str(exe), str(tmp_path / "g.dat"), "5", "--json", "--repeat", "3"], capture_output=True,
                       text=True)
    line = [l for l in clean(r.stdout).splitlines() if l.startswith("{")]
    import json
    j = json.loads(line[0])
    want = oracle.bfs(g.offsets, g.cols, 5)
    assert j["source"] == 5 and j["depth"] == int(want.max()) and j["repeat"] == 3 and j["errors"] == 0
    assert j["edges"] == oracle.reached_edges(g.offsets, want)


def test_interactive_loop(exe, tmp_path):
    g = d.gen_rmat(10, 8, seed=53)
    g.save(tmp_path / "g.dat", "dat")
    s = g.pick_sources(2, seed=53).tolist()
    stdin = f"n\n{s[0]}\nn\n{g.n + 3}\n{s[1]}\ny\n"
    r = subprocess.run([str(exe), str(tmp_path / "g.dat"), "$"], input=stdin, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # prompts do not echo the typed source; the depths show which sources ran (an out-of-range one is
    # asked again)
    assert field(r.stdout, r"Source  : (\d+)") == [str(g.source)]
    assert field(r.stdout, r"- Error = (\d+)") == ["0", "0", "0"]
    dists = field(r.stdout, r"- Dist  = (\d+)")
    assert dists == [str(oracle.bfs(g.offsets, g.cols, x).max()) for x in (g.source, s[0], s[1])]
    assert "Exit? [y/n]" in r.stdout


@pytest.mark.parametrize("tiles,grid", [(None, None), ((8, 64, 1024, 16384), 72)])
def test_frontier_profile_lines(exe, tmp_path, tiles, grid):
    g = d.gen_rmat(12, 16, seed=54)
    g.source = int(g.pick_sources(1, seed=54)[0])
    g.save(tmp_path / "g.dat", "dat")
    args = [str(exe), str(tmp_path / "g.dat"), "--frontier-profile"]
    if tiles:
        args += ["--profile-tiles", ",".join(map(str, tiles)), "--profile-grid", str(grid)]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    tiles = tiles or (16, 128, 1024, 8192)
    grid = grid or 304
    text = clean(r.stdout)
    assert f"Dim: {grid} 1024" in text
    assert f"Siz: {' '.join(map(str, tiles))} {grid * 1024}" in text
    assert f"Rng: {' '.join(map(str, tiles))} inf" in text
    rows = [list(map(int, m.groups())) for m in re.finditer(r"^(\d+): (\d+) (\d+) (\d+) (\d+) (\d+)$", text, re.M)]
    want = oracle.bfs(g.offsets, g.cols, g.source)
    idle, _ = d.frontier_profile(g, want, tiles, grid * 1024)
    assert [row[0] for row in rows] == list(range(len(idle)))
    assert np.array_equal(np.array([row[1:] for row in rows], np.int64), idle)
    assert text.index("Rng:") < text.index("- Dist")
    assert r.stdout.split()[-2] == "0.125ms"


def test_hub_first_renumbering_on_the_host(tmp_path):
    """dfq::hub_first_csr (pools renumber wide skewed graphs with it): a C++
    check of its properties, built against the library's host sources."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = tmp_path / "hub_first_check"
    srcs = [CSRC / "host_graph.cpp", CSRC / "host_gen.cpp", ROOT / "tests" / "cli_double" / "hub_first_check.cpp"]
    subprocess.run([cxx, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{CSRC}", *map(str, srcs), "-o", str(out),
                    "-pthread"], check=True)
    r = subprocess.run([str(out)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_opt_names(exe, tmp_path):
    """--opt takes every kernel-shape field by name (the device double ignores
    them) and rejects unknown names before loading anything."""
    g = d.gen_rmat(10, 8, seed=53)
    g.source = int(g.pick_sources(1, seed=53)[0])
    g.save(tmp_path / "g.dat", "dat")
    args = [str(exe), str(tmp_path / "g.dat")]
    for kv in ("cluster_blocks=8", "direction=0", "probe_first=1", "block_threads=1024"):
        r = subprocess.run(args + ["--opt", kv], capture_output=True, text=True)
        assert r.returncode == 0, (kv, r.stderr)
        assert field(r.stdout, r"- Error = (\d+)") == ["0"]
    r = subprocess.run(args + ["--opt", "no_such_field=1"], capture_output=True, text=True)
    assert r.returncode == 2 and "dfq_opts field" in r.stderr
