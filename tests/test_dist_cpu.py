"""The multi-process path of bench.py on CPU (gloo, world size 2): the
barrier, the max-over-ranks time and the whole-job edge sum that replicas
report, and the reference arm running on rank 0 only.  Single-source BFS does
not shard, so N GPUs run N replicas; no data-path collective exists."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r'''
import os, sys, json
sys.path[:0] = [{root!r} + "/dfq-bfs_gb300", {root!r}]
import bench
ws, rank, local, pg = bench.dist_setup(2)
bench.barrier(pg)
t = bench.allreduce_max(pg, 1.5 + rank)       # per-rank step time
e = bench.allreduce_sum(pg, 100.0 * (rank + 1))  # per-rank edges
bench.barrier(pg)
print(json.dumps({{"rank": rank, "ws": ws, "max": t, "sum": e}}))
pg.destroy_process_group()
'''


def run_ranks(code: str, port: int, extra_env=None, args=()):
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", code, *args], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    return procs, outs


def test_gloo_replica_reductions():
    pytest.importorskip("torch.distributed")
    procs, outs = run_ranks(WORKER.format(root=str(ROOT)), free_port())
    import json
    res = sorted((json.loads(o[0].strip().splitlines()[-1]) for o in outs), key=lambda r: r["rank"])
    for p, o in zip(procs, outs):
        assert p.returncode == 0, o[1]
    assert [r["ws"] for r in res] == [2, 2]
    assert all(r["max"] == 2.5 for r in res)    # slowest rank's time
    assert all(r["sum"] == 300.0 for r in res)  # whole-job work


def test_reference_arm_rank0_only(tmp_path):
    """bench.py --impl reference under two ranks: rank 0 prints the line,
    rank 1 exits 0 without work (a small R-MAT scale keeps it quick).  The
    arm builds its workload through the oracle alone: the product library is
    never loaded in that process."""
    pytest.importorskip("torch.distributed")
    code = (f"import sys; sys.path[:0]=[{str(ROOT)!r}+'/dfq-bfs_gb300', {str(ROOT)!r}]; "
            "import bench; "
            "sys.argv=['bench.py','--impl','reference','--gpus','2','--steps','2','--warmup','1','--scale','10']; "
            "rc = bench.main(); "
            "assert 'dfqbfs' not in sys.modules; "
            "assert not [l for l in open('/proc/self/maps') if 'libdfq' in l]; "
            "sys.exit(rc)")
    procs, outs = run_ranks(code, free_port())
    for p, o in zip(procs, outs):
        assert p.returncode == 0, o[1]
    lines = [o[0].strip() for o in outs]
    import json
    line = json.loads(lines[0].splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert lines[1] == ""
