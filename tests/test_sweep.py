"""The plot.py-compatible sweep runner (CPU): output parsing, averaging,
result.csv layout, variant wrappers, and bfs --opt argument checking."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

from dfqbfs import sweep

ROOT = Path(__file__).resolve().parent.parent


def fake_program(path: Path, times):
    """A stand-in program printing the reference's stdout block with the given
    times in turn (a counter file keeps the position)."""
    counter = path.with_suffix(".n")
    body = (f"#!{sys.executable}\n"
            "import sys, pathlib\n"
            f"c = pathlib.Path({str(counter)!r}); k = int(c.read_text()) if c.exists() else 0\n"
            f"t = {list(times)!r}[k % {len(times)}]; c.write_text(str(k + 1))\n"
            "print('\\033[0;1;33mx\\033[0;1m'); print('# Nodes : 3'); print('# Edges : 2'); print('Source  : 0')\n"
            "print('- Dist  = 1'); print('- Touch = 100 % (3 / 3)'); print('- Error = 0')\n"
            "print(f'- Time  = {t:.6f}ms'); print('\\033[0m')\n")
    path.write_text(body)
    path.chmod(0o755)


def test_parse_time_like_plot_py():
    out = "banner\n# Nodes : 5\n- Error = 0\n- Time  = 12.500000ms\n\x1b[0m\n"
    assert sweep.parse_time_ms(out) == 12.5
    with pytest.raises(ValueError):
        sweep.parse_time_ms("no time here")


def test_sweep_means_and_csv_layout(tmp_path):
    data = tmp_path / "data"
    bins = tmp_path / "bin"
    data.mkdir()
    bins.mkdir()
    (data / "g2.dat").write_text("x")
    (data / "g1.dat").write_text("x")
    fake_program(bins / "b_fast", [1.0, 3.0])
    fake_program(bins / "a_slow", [10.0])
    names, graphs, m = sweep.run_sweep(2, data, bins, log=lambda *a: None)
    assert names == ["a_slow", "b_fast"] and graphs == ["g1.dat", "g2.dat"]
    assert m == [[10.0, 10.0], [2.0, 2.0]]
    csv_path = tmp_path / "result.csv"
    sweep.write_csv(csv_path, names, graphs, m)
    lines = csv_path.read_text().splitlines()
    assert lines[0] == "\tbenchmark\ta_slow\tb_fast"
    assert lines[1].split("\t")[:2] == ["0", "g1.dat"] and float(lines[1].split("\t")[3]) == 2.0
    assert sweep.read_csv(csv_path) == (names, graphs, m)


def test_sweep_reports_failing_program(tmp_path):
    (tmp_path / "data").mkdir()
    (tmp_path / "bin").mkdir()
    (tmp_path / "data" / "g").write_text("x")
    bad = tmp_path / "bin" / "bad"
    bad.write_text("#!/bin/sh\nexit 3\n")
    bad.chmod(0o755)
    with pytest.raises(RuntimeError, match="exited 3"):
        sweep.run_sweep(1, tmp_path / "data", tmp_path / "bin", log=lambda *a: None)


def test_make_variants_and_cli(tmp_path):
    made = sweep.make_variants(tmp_path / "bin", bfs=Path("/opt/x/bfs"))
    assert {p.name for p in made} == set(sweep.VARIANTS)
    body = (tmp_path / "bin" / "dfq_claim_at_once").read_text()
    assert "--opt probe_first=0" in body and "--ref-compat" in body and os.access(made[0], os.X_OK)
    rc = subprocess.run([sys.executable, "-m", "dfqbfs.sweep", "--make-variants", str(tmp_path / "v")],
                        cwd=ROOT / "dfq-bfs_gb300", capture_output=True, text=True)
    assert rc.returncode == 0 and len(list((tmp_path / "v").iterdir())) == len(sweep.VARIANTS)


def test_bfs_rejects_bad_opt(tmp_path):
    """bfs checks --opt before it touches the graph or the GPU."""
    exe = ROOT / "dfq-bfs_gb300" / "bin" / "bfs"
    if not exe.exists():
        pytest.skip("bfs not built")
    for bad in ["nonsense=1", "probe_first", "probe_first=x"]:
        p = subprocess.run([str(exe), str(tmp_path / "none.dat"), "--opt", bad], capture_output=True, text=True)
        assert p.returncode == 2 and "--opt" in p.stderr
