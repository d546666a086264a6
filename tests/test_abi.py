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


def test_option_struct_layout_matches_header():
    """The ctypes mirror of dfq_opts has the header's int32 fields in the
    header's order (a mismatch would shift every option after it)."""
    assert [f for f, _ in d.Opts._fields_] == struct_fields("dfq_opts")
    assert all(t is C.c_int32 for _, t in d.Opts._fields_)
    o = d.default_opts()
    assert o.stall_test_level == 0 and o.direction == 0 and o.timeout_ms == 5000


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
    assert o.block_threads in (256, 512, 1024) and o.large_min_degree >= 32
    assert d.lib().dfq_graph_num_vertices(None) == -1


def test_bfs_program_usage():
    exe = ROOT / "dfq-bfs_gb300" / "bin" / "bfs"
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([str(exe), "/nonexistent.dat"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
