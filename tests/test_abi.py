"""The C ABI (CPU only): the library loads, exports every declared symbol,
and rejects bad arguments before touching a device."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import dfqbfs as d

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "dfq.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dfq_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert sorted(d.EXPORTS) == declared_functions()


def struct_fields(name):
    """Field names of `typedef struct name {...} name;` in dfq.h, in order."""
    text = (ROOT / "include" / "dfq.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, flags=re.S).group(1)
    return re.findall(r"\b(?:u?int(?:8|16|32|64)_t|double|float)\s+(\w+)\s*;", body)


MIRRORS = {"dfq_csr": "_Csr", "dfq_opts": "Opts", "dfq_stats": "Stats", "dfq_level_info": "LevelInfo",
           "dfq_query": "Query", "dfq_query_result": "QueryResult", "dfq_server_opts": "ServerOpts",
           "dfq_server_result": "ServerResult"}


def test_option_struct_layout_matches_header():
    """The ctypes mirror of dfq_opts has the header's int32 fields in the
    header's order (a mismatch would shift every option after it)."""
    assert [f for f, _ in d.Opts._fields_] == struct_fields("dfq_opts")
    assert all(t is C.c_int32 for _, t in d.Opts._fields_)
    o = d.default_opts()
    assert o.stall_test_level == 0 and o.direction == 0 and o.timeout_ms == 5000
    assert o.cluster_blocks == 0 and o.probe_first == 2 and o.block_threads == 0


def test_struct_mirrors_match_the_c_layout(tmp_path):
    """Every struct the binding mirrors has the C compiler's size and field
    offsets (a C program built against dfq.h prints them)."""
    import shutil
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dfq.h"', "int main(void) {"]
    for cname, pyname in MIRRORS.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in getattr(d, pyname)._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, f, v = line.split()
        got[(cname, f)] = int(v)
    for cname, pyname in MIRRORS.items():
        cls = getattr(d, pyname)
        assert C.sizeof(cls) == got[(cname, "sizeof")], cname
        for f, _ in cls._fields_:
            assert getattr(cls, f).offset == got[(cname, f)], (cname, f)


def test_library_exports_every_declared_symbol():
    L = d.lib()
    for name in declared_functions():
        assert hasattr(L, name), name


def test_no_oracle_in_product():
    """The product library neither links nor names the oracle."""
    lib = (ROOT / "dfq-bfs_gb300" / "lib" / "libdfq.so").read_bytes()
    assert b"oracle_" not in lib and b"liboracle" not in lib
    for src in (ROOT / "dfq-bfs_gb300").rglob("*"):
        if src.suffix in (".py", ".cpp", ".cu", ".cuh", ".hpp", ".h"):
            assert "import oracle" not in src.read_text() and "oracle/" not in src.read_text(), src


def test_bad_arguments():
    L = d.lib()
    h = C.c_void_p()
    assert L.dfq_graph_create(None, None, 0, 0, None, C.byref(h)) == -1
    assert b"need offsets" in L.dfq_last_error()
    assert L.dfq_bfs(None, 0, None, None, None) == -1
    assert L.dfq_graph_destroy(None) == -1
    o = d.default_opts()
    assert o.block_threads in (0, 256, 512, 1024) and o.large_min_degree >= 32
    assert d.lib().dfq_graph_num_vertices(None) == -1


def test_bfs_program_usage():
    exe = ROOT / "dfq-bfs_gb300" / "bin" / "bfs"
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([str(exe), "/nonexistent.dat"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
    # profile options are checked before anything is loaded
    r = subprocess.run([str(exe), "/nonexistent.dat", "--frontier-profile", "--profile-tiles", "16,100,1024,8192"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "powers of two" in r.stderr
    r = subprocess.run([str(exe), "/nonexistent.dat", "--profile-grid", "0"], capture_output=True, text=True)
    assert r.returncode == 2 and "block count" in r.stderr
