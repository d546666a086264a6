#!/usr/bin/env python3
"""Benchmark: single-source BFS on RMAT scale 22 (edge factor 16, a/b/c/d =
.57/.19/.19/.05, symmetrised, deduplicated, no self-loops, seeded), 64 seeded
non-isolated sources run one at a time.

One step = 64 BFS launches, one per source, with the graph resident in HBM.
  value  GTEPS = sum over the step's BFS of E_R (out-degrees of reached
         vertices) / device time of the step (CUDA events on the graph's
         stream, synchronize on both sides), levels written to device buffers.
  e2e    the same metric through the public C ABI call dfq_bfs() with HOST
         (pinned) level buffers: launch + device->host copy of every level
         array inside the timed region.
  roofline  algorithmic bytes per BFS = 4*E_R + 8*|R| + 4*N over the average
         launch time of the BFS kernel (events around each launch), against
         the measured HBM copy bandwidth.
  parity every timed source's levels (from the untimed counter pass) against
         the oracle, bit for bit, with the kernel's E_R; outside the timed region.
  cpu_baseline  the oracle (the reference's serial CPU BFS, restated in C) on
         a bounded sample of the sources, 1 host core (host CPU model and
         core count reported beside it).
  reference_gpu the reference's own kernel (design/shared-q/atomic-sa/our-sep/
         upper-bound/bfs.cu) compiled from its sources, same graph and
         sources, its "- Time" definition.

--impl reference: the reference's CPU path (the oracle port; the reference's
serial BFS is inlined in its main() and cannot be built alone) on the same
workload, one source per step.  Its graph and sources come from the oracle's
restated generator (oracle/gen.c, byte-identical to the product's), so that
process never loads the product library; its config equals this arm's.
Multi-GPU (torchrun): replicas only - each rank runs the full step on its own
copy of the graph (weak scaling); value sums all ranks' edges over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT / "dfq-bfs_gb300"), str(ROOT)]

import numpy as np  # noqa: E402

METRIC = "BFS GTEPS (RMAT-22 EF16, 64 sources one at a time)"
UNIT = "GTEPS"
WORKLOAD = {"workload": "rmat22_ef16_64src", "graph": "RMAT scale 22, edge factor 16, a=.57 b=.19 c=.19 d=.05",
            "symmetrized": True, "dedup": True, "self_loops": False, "seed": 1, "sources": 64,
            "source_seed": 1, "l2": "inputs larger than L2 (column array ~0.5 GB > 129 MB L2)"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        j = json.loads(p.read_text())
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def host_cpu() -> dict:
    """Model name and logical core count of this host (reported beside every CPU baseline)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not model:
        try:
            for line in Path("/proc/cpuinfo").read_text().splitlines():
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    import platform
    return {"model": model or platform.processor() or platform.machine(), "nproc": os.cpu_count(),
            "arch": platform.machine()}


def oracle_parity(offsets, cols, sources, device_levels, device_er=None, threads=None) -> dict:
    """Bit-exact comparison of device level arrays with the serial oracle BFS
    (the reference's own per-run check, applied to every source), run on the
    host's cores (ctypes releases the GIL during each oracle call).
    device_levels(i) returns source i's level array as numpy; device_er[i], if
    given, is the kernel's E_R for source i, checked against the oracle's."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    oracle.lib()
    t0 = time.perf_counter()
    bad, er_bad, first = 0, 0, None
    with ThreadPoolExecutor(max_workers=threads or min(16, os.cpu_count() or 1)) as ex:
        futs = [ex.submit(oracle.bfs, offsets, cols, int(s)) for s in sources]
        for i, f in enumerate(futs):
            want = f.result()
            got = device_levels(i)
            mm = oracle.compare(want, got)["mismatches"]
            if mm and first is None:
                first = {"source": int(sources[i]), "mismatches": int(mm)}
            bad += int(mm != 0)
            if device_er is not None and int(device_er[i]) != oracle.reached_edges(offsets, want):
                er_bad += 1
            futs[i] = None
    out = {"sources_checked": len(sources), "mismatches": bad, "oracle_s": round(time.perf_counter() - t0, 1)}
    if device_er is not None:
        out["edge_count_mismatches"] = er_bad
    if first:
        out["first_mismatch"] = first
    return out


def load_graph(scale: int = 22):
    import dfqbfs as d
    cache = Path(os.environ.get("DFQ_BENCH_CACHE", "/tmp")) / f"dfq_rmat{scale}_ef16_s1.bin"
    if cache.exists():
        try:
            return d.load(cache, "bin")
        except d.DfqError:
            pass
    g = d.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=1)
    try:
        g.save(cache, "bin")
    except d.DfqError:
        pass
    return g


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                out, _ = self.p.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce_max(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def cpu_sample(g, sources, budget_s=15.0):
    """Oracle BFS (1 core) over sources until ~budget_s of CPU work."""
    import oracle
    edges, t_total, done = 0, 0.0, 0
    for s in sources:
        t0 = time.perf_counter()
        lv = oracle.bfs(g.offsets, g.cols, int(s))
        t_total += time.perf_counter() - t0
        edges += oracle.reached_edges(g.offsets, lv)
        done += 1
        if t_total >= budget_s:
            break
    return edges, t_total, done


def reference_workload(scale: int = 22):
    """The headline graph and sources built through the oracle's restated
    generator (byte-identical to the product's, tests/test_oracle_gen.py), so
    that the reference arm never loads the product library."""
    import oracle
    off, cols = oracle.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=1)
    srcs = oracle.pick_sources(off, 64, seed=1)
    return off, cols, srcs


def run_reference(args, ws, rank, pg):
    """The reference's CPU path - its serial BFS (bfs.cu:216-253), restated in
    oracle/oracle.c because the reference inlines it in a main() built on
    managed GPU memory - on all the host's threads: each step runs one source
    per thread side by side (each search serial, like the reference's), and
    the value is the edges of all of them over the step's wall time.  Graph
    and sources come from oracle/gen.c."""
    if rank != 0:
        return 0
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    t_gen = time.perf_counter()
    off, cols, srcs = reference_workload(args.scale)
    t_gen = time.perf_counter() - t_gen
    n, e = len(off) - 1, len(cols)
    threads = max(1, os.cpu_count() or 1)
    oracle.lib()

    def one(s):  # the oracle's C calls release the GIL
        return oracle.reached_edges(off, oracle.bfs(off, cols, int(s)))

    def batch(step):
        return [int(srcs[(step * threads + k) % len(srcs)]) for k in range(threads)]

    edges, ts = 0, []
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for i in range(args.warmup):
            list(ex.map(one, batch(i)))
        for i in range(args.steps):
            b = batch(args.warmup + i)
            t0 = time.perf_counter()
            got = list(ex.map(one, b))
            ts.append(time.perf_counter() - t0)
            edges += sum(got)
    tot = sum(ts)
    val = edges / tot / 1e9
    metric = METRIC if args.scale == 22 else f"BFS GTEPS (RMAT-{args.scale} EF16, 64 sources one at a time)"
    line = {"metric": metric, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
            "config": workload_config(n, e, ws), "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} steps of {threads} of the 64 sources side by side "
                                       f"(one serial oracle BFS per host thread)",
                             "host": host_cpu()},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gen_s": round(t_gen, 1)}
    print(json.dumps(line))
    return 0


def workload_config(n: int, e: int, ws: int) -> dict:
    """The headline workload's config, identical in both arms."""
    return dict(WORKLOAD, n=int(n), e=int(e), parallelism=f"replicas x{ws}")


def pool256_graphs(seed: int = 1, count: int = 256):
    """The 256-graph batch pool: 3/4 R-MAT (scale uniform in 10..20, edge factor 8, 16
    or 32, symmetrised, deduplicated) and 1/4 grids (side log-uniform in
    64..1024, 1% of edges deleted, largest component), each seeded by its
    index.  Generated on several host threads (each generator call releases
    the GIL) and cached as binary CSR in DFQ_BENCH_CACHE (default /tmp)."""
    import dfqbfs as d
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(seed)
    cache = Path(os.environ.get("DFQ_BENCH_CACHE", "/tmp")) / f"dfq_pool256_s{seed}"
    cache.mkdir(parents=True, exist_ok=True)
    specs = []
    for i in range(count):
        if i % 4 != 3:
            specs.append(("rmat", int(rng.integers(10, 21)), int(rng.choice([8, 16, 32]))))
        else:
            specs.append(("grid", int(round(64 * 2 ** rng.uniform(0, 4))), 0))

    def make(i):
        kind, a, b = specs[i]
        f = cache / f"g{i}_{kind}_{a}_{b}.bin"
        if f.exists():
            try:
                return d.load(f, "bin")
            except d.DfqError:
                pass
        g = d.gen_rmat(a, b, seed=1000 + i) if kind == "rmat" else d.gen_grid(a, 0.01, seed=1000 + i)[0]
        try:
            g.save(f, "bin")
        except d.DfqError:
            pass
        return g

    # largest first, so the long generations overlap
    order = sorted(range(count), key=lambda i: -(specs[i][1] if specs[i][0] == "rmat" else 0))
    graphs = [None] * count
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        for i, g in zip(order, ex.map(make, order)):
            graphs[i] = g
    return graphs, specs


def kernel_opts(d, args):
    """Default dfq_opts with the --opt NAME=VALUE overrides applied."""
    o = d.default_opts()
    for kv in args.opt:
        k, v = kv.split("=", 1)
        setattr(o, k, int(v))
    return o


def batch_record(torch, d, steps: int, warmup: int, sizes=(64, 128, 256, 512, 1024), spot: int = 32,
                 opts=None, tune: bool = False) -> dict:
    """The batched configuration: 1024 queries (4 seeded sources per graph) over
    the 256-graph pool, compared with one plain cooperative launch per query
    at matched latency.

    Latency is service latency on both sides, with no host queueing: a plain
    query's is its own launch (events around it); a batched query's is the
    time from its batch's launch start to its completion on the device clock
    (every query of the batch is submitted at that start).  The queries, in a
    seeded shuffled order, run as consecutive batches of each size; a size's
    queries/s is its queries over the sum of its batch times.  `at_equal_p99`
    is the largest size whose p99 does not exceed the plain launches' p99, with
    its queries/s over the plain launches' (1024 queries launched back to back)."""
    import oracle
    t_gen = time.perf_counter()
    graphs, specs = pool256_graphs()
    t_gen = time.perf_counter() - t_gen
    pool = d.Pool(graphs, opts if opts is not None else d.default_opts())
    try:
        queries = []
        for gi, g in enumerate(graphs):
            for s in g.pick_sources(4, seed=gi):
                queries.append((gi, int(s), torch.empty(g.n, dtype=torch.int32, device="cuda")))
        nq = len(queries)
        tuned = None
        if tune:  # dfq_pool_autotune on the full batch, then everything below runs tuned
            base_opts = pool.opts().as_dict()
            for _ in range(2):
                pool.batch(queries, 0)
            t0 = time.perf_counter()
            _, ms0 = pool.batch(queries, 0)
            best = pool.autotune(queries)
            tuned = {"default_opts": base_opts, "tuned_opts": best.as_dict(),
                     "tune_s": round(time.perf_counter() - t0, 1), "full_batch_ms_default": ms0}
        nwide = sum(1 for q in queries if pool.info(q[0])[2])
        # query kinds as the batch kernel splits them: wide graphs on the
        # whole grid, large high-diameter graphs on gangs, the rest on a block
        kind = []
        for q in queries:
            n_, e_, w_ = pool.info(q[0])
            kind.append("wide" if w_ else "gang" if (n_ >= 65536 and e_ < 8 * n_) else "narrow")
        order = np.random.default_rng(11).permutation(nq)
        # plain launches, one per query (each its own cooperative launch)
        for q in queries[:8]:
            pool.bfs(q[0], q[1], q[2])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain_ms = [pool.bfs(q[0], q[1], q[2]).kernel_ms for q in queries]
        plain_total_s = time.perf_counter() - t0
        kinds_all = np.array(kind)
        pm = np.array(plain_ms)
        plain = {"queries_per_s": nq / plain_total_s, "p50_ms": float(np.percentile(plain_ms, 50)),
                 "p99_ms": float(np.percentile(plain_ms, 99)), "total_ms": plain_total_s * 1e3,
                 "p99_ms_by_kind": {kd: float(np.percentile(pm[kinds_all == kd], 99))
                                    for kd in ("wide", "gang", "narrow") if (kinds_all == kd).any()}}
        per_size, edges_all = [], 0
        for bs in sizes:
            groups = [[queries[k] for k in order[i:i + bs]] for i in range(0, nq, bs)]
            # one batch shape: replay a captured CUDA graph; several shapes:
            # plain launches (a re-capture would sit inside the timed events)
            flags = d.BATCH_GRAPH if len(groups) == 1 else 0
            for _ in range(max(warmup, 1)):
                for grp in groups:
                    pool.batch(grp, flags)
            lat, tot_ms = [], []
            for _ in range(max(steps, 1)):
                ms_step, lat_step = 0.0, []
                for grp in groups:
                    res, dev_ms = pool.batch(grp, flags)
                    ms_step += dev_ms
                    lat_step += [r.end_us / 1e3 for r in res]
                    if bs == sizes[-1]:
                        edges_all = sum(r.edges for r in res)
                tot_ms.append(ms_step)
                lat.append(lat_step)
            ms = float(np.median(tot_ms))
            lat = np.median(np.array(lat), axis=0)
            kinds = np.array([kind[k] for k in order])  # queries in the order the batches ran them
            per_size.append({"batch": bs, "launches": len(groups), "cuda_graph": flags != 0,
                             "queries_per_s": nq / (ms * 1e-3),
                             "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                             "p99_ms_by_kind": {kd: float(np.percentile(lat[kinds == kd], 99))
                                                for kd in ("wide", "gang", "narrow") if (kinds == kd).any()},
                             "ms_all": ms})
        # parity: `spot` queries of the last batches against the oracle
        rng = np.random.default_rng(3)
        bad = 0
        for k in rng.choice(nq, size=min(spot, nq), replace=False):
            gi, s, lv = queries[k]
            bad += int(not np.array_equal(lv.cpu().numpy(), oracle.bfs(graphs[gi].offsets, graphs[gi].cols, s)))
        ok = [r for r in per_size if r["p99_ms"] <= plain["p99_ms"]]
        eq = max(ok, key=lambda r: r["batch"]) if ok else None
        full = per_size[-1]
        return {"workload": "batch_256graphs_1024q", "graphs": len(graphs),
                "rmat": sum(1 for sp in specs if sp[0] == "rmat"), "grids": sum(1 for sp in specs if sp[0] == "grid"),
                "queries": nq, "wide_queries": nwide, "total_edges": int(sum(g.e for g in graphs)),
                "gen_s": round(t_gen, 1), "per_query_plain": plain, "batched": per_size, "autotune": tuned,
                "kernel_opts": pool.opts().as_dict(),
                "speedup_qps_full_batch": full["queries_per_s"] / plain["queries_per_s"],
                "at_equal_p99": ({"batch": eq["batch"], "queries_per_s": eq["queries_per_s"], "p99_ms": eq["p99_ms"],
                                  "speedup_qps": eq["queries_per_s"] / plain["queries_per_s"]} if eq else None),
                "gteps_full_batch": edges_all / (full["ms_all"] * 1e-3) / 1e9,
                "parity_spot_check": {"queries": min(spot, nq), "mismatches": bad},
                "latency": "service latency: plain = the query's own launch; batched = from its batch's launch "
                           "start to its completion (all queries of a batch submitted at that start)"}
    finally:
        pool.close()


def run_batch(args, torch, d):
    """Batched workload line: queries/s of the full 1024-query batch, with the
    matched-latency comparison against per-query plain launches."""
    rec = batch_record(torch, d, args.steps, args.warmup, opts=kernel_opts(d, args), tune=args.pool_autotune)
    full = rec["batched"][-1]
    out = {"metric": "batched BFS queries/s (1024 queries over 256 graphs)", "value": full["queries_per_s"],
           "unit": "queries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": full["ms_all"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded)", "config": {"workload": rec["workload"], "graphs": rec["graphs"],
                                                    "queries": rec["queries"]}, "batch": rec}
    print(json.dumps(out))
    return 0


def serve_pool(target_gb: float = 40.0):
    """The serving pool: R-MAT scales 16..24 (edge factor 16) and grids with
    sides 1024, 2048, 4096 (1% deleted, largest component), each generated
    once and uploaded as many times as it takes to hold ~target_gb of CSR on
    the device (the copies are separate device graphs)."""
    import dfqbfs as d
    cache = Path(os.environ.get("DFQ_BENCH_CACHE", "/tmp")) / "dfq_serve_pool"
    cache.mkdir(parents=True, exist_ok=True)
    specs = [("rmat", s) for s in range(16, 25)] + [("grid", side) for side in (1024, 2048, 4096)]
    distinct = []
    for kind, a in specs:
        f = cache / f"{kind}_{a}.bin"
        g = None
        if f.exists():
            try:
                g = d.load(f, "bin")
            except d.DfqError:
                g = None
        if g is None:
            g = d.gen_rmat(a, 16, seed=2000 + a) if kind == "rmat" else d.gen_grid(a, 0.01, seed=3000 + a)[0]
            g.save(f, "bin")
        distinct.append(g)
    gb = sum(4 * (g.n + 1 + g.e) for g in distinct) / 1e9
    replicas = max(1, int(round(target_gb / gb)))
    return distinct, specs, replicas, gb


def run_serve(args, torch, d):
    """Serving workload: Poisson request streams at swept rates over a ~40 GB resident
    pool, served by the continuous-batching server (trace replay in C++)."""
    import oracle
    t_gen = time.perf_counter()
    distinct, specs, replicas, gb = serve_pool()
    t_gen = time.perf_counter() - t_gen
    pool_graphs = [g for _ in range(replicas) for g in distinct]
    t_up = time.perf_counter()
    pool = d.Pool(pool_graphs, kernel_opts(d, args))
    t_up = time.perf_counter() - t_up
    kopts = pool.opts().as_dict()
    free_b, _ = torch.cuda.mem_get_info()
    budget = int(min(48e9, free_b * 0.5))
    srv = d.Server(pool, hbm_budget_bytes=budget, ring_capacity=8192, idle_ms=20)
    cand = [g.pick_sources(256, seed=i) for i, g in enumerate(distinct)]
    rng = np.random.default_rng(5)
    rates = [int(x) for x in args.rates.split(",")]
    per_rate = []
    for rate in rates:
        n = int(min(rate * args.serve_seconds, args.serve_max))
        arr = np.cumsum(rng.exponential(1e6 / rate, size=n))
        gi = rng.integers(0, len(pool_graphs), size=n)
        src = np.array([cand[g % len(distinct)][rng.integers(0, 256)] for g in gi], np.int32)
        # spot checks: a few requests on graphs the oracle handles quickly
        small = [i for i in range(n) if pool_graphs[gi[i]].e < 40_000_000]
        keep = np.zeros(n, np.int32)
        for i in rng.choice(small, size=min(4, len(small)), replace=False):
            keep[i] = 1
        t0 = time.perf_counter()
        res = srv.replay(gi, src, arr, keep)
        wall = time.perf_counter() - t0
        lat = np.array([r.done_us - r.submit_us for r in res]) / 1e3
        span = (max(r.done_us for r in res) - arr[0]) / 1e6
        bad = 0
        for i in np.flatnonzero(keep):
            g = pool_graphs[gi[i]]
            lv, _ = srv.levels(res[i].id, g.n)
            bad += int(not np.array_equal(lv, oracle.bfs(g.offsets, g.cols, int(src[i]))))
            srv.release(res[i].id)
        per_rate.append({"offered_qps": rate, "requests": n, "sustained_qps": n / span,
                         "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                         "max_ms": float(lat.max()), "wide_share": float(np.mean([r.wide for r in res])),
                         "retried": int(sum(r.retried for r in res)), "errors": int(sum(r.status != 0 for r in res)),
                         "gteps": float(sum(r.edges for r in res) / span / 1e9), "wall_s": round(wall, 2),
                         "spot_checks": int(keep.sum()), "spot_mismatches": bad})
    srv.close()
    pool.close()
    best = max(per_rate, key=lambda x: x["sustained_qps"])
    out = {"metric": "BFS serving sustained queries/s (Poisson arrivals, ~40 GB pool)",
           "value": best["sustained_qps"], "unit": "queries/s", "n_gpus": 1, "steps": len(rates), "warmup": 0,
           "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded)",
           "kernel_opts": kopts,
           "config": {"workload": "serve_poisson_40gb", "distinct_graphs": [f"{k}{a}" for k, a in specs],
                      "replicas": replicas, "pool_graphs": len(pool_graphs), "pool_gb": round(gb * replicas, 1),
                      "hbm_budget_gb": round(budget / 1e9, 1), "queries": "uniform over pool graphs, uniform "
                      "non-isolated sources", "gen_s": round(t_gen, 1), "upload_s": round(t_up, 1)},
           "per_rate": per_rate}
    print(json.dumps(out))
    return 0


def grid_sources(orig, side: int, k_interior: int = 12, seed: int = 1):
    """Grid-workload sources: the 4 corners of the full grid (nearest kept vertex if
    a corner left the largest component) and k seeded interior vertices."""
    pos = {int(f): i for i, f in enumerate(orig)} if len(orig) < 1 << 22 else None
    lookup = (lambda f: pos.get(f)) if pos is not None else (
        lambda f: (lambda j: int(j) if j < len(orig) and orig[j] == f else None)(np.searchsorted(orig, f)))
    out = []
    for r0, c0 in [(0, 0), (0, side - 1), (side - 1, 0), (side - 1, side - 1)]:
        found = None
        for rad in range(side):
            for dr in range(-rad, rad + 1):
                for dc in (-(rad - abs(dr)), rad - abs(dr)):
                    r, c = r0 + dr, c0 + dc
                    if 0 <= r < side and 0 <= c < side:
                        v = lookup(r * side + c)
                        if v is not None:
                            found = v
                            break
                if found is not None:
                    break
            if found is not None:
                break
        out.append(found)
    rng = np.random.default_rng(seed)
    interior = rng.choice(len(orig), size=k_interior, replace=False)
    return out + [int(x) for x in interior]


def workload_graph(name: str, scale: int):
    import dfqbfs as d
    if name == "rmat22":
        g = load_graph(scale)
        return g, g.pick_sources(64, seed=1), dict(WORKLOAD, n=int(g.n), e=int(g.e))
    if name == "grid4096":
        g, orig = d.gen_grid(4096, 0.01, seed=1)
        srcs = np.array(grid_sources(orig, 4096), np.int32)
        return g, srcs, {"workload": "grid4096_del1pct_lcc_16src", "graph": "4096x4096 4-neighbour grid, 1% of "
                         "undirected edges deleted (seeded), largest component, row-major relabel", "seed": 1,
                         "sources": 16, "n": g.n, "e": g.e}
    if name == "zipf262k":
        g = d.gen_zipf_geometric(262144, 4.7, 2.1, seed=1)
        return g, np.array([0], np.int32), {"workload": "zipf_geometric_262144_src0", "n": g.n, "e": g.e}
    raise SystemExit(f"unknown workload {name}")


def measure_device(dg, srcs, n, steps, warmup, torch, with_clocks=None, keep_levels=False):
    """Device-resident timing of `steps` passes over srcs (one launch per
    source); returns total ms (events on the graph's stream), per-launch ms,
    per-source E_R / |R| / levels, and with keep_levels each source's level
    array from the untimed pass (host copies, for the oracle check)."""
    stream = torch.cuda.ExternalStream(dg.stream)
    levels = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(2)]
    er, rr, lvls, host_levels = [], [], [], []
    for s in srcs:  # untimed pass: E_R and |R| from the kernel's own counters
        dg.launch(int(s), levels[0])
        st = dg.last_stats()
        er.append(st.edges)
        rr.append(st.reached)
        lvls.append(st.levels)
        if keep_levels:
            host_levels.append(levels[0].cpu().numpy())

    def step(evs=None):
        for i, s in enumerate(srcs):
            if evs is not None:
                evs[i][0].record(stream)
            dg.launch(int(s), levels[i & 1])
            if evs is not None:
                evs[i][1].record(stream)

    for _ in range(warmup):
        step()
    dg.sync()
    evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in srcs]
           for _ in range(steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if with_clocks is not None:
        with_clocks.__enter__()
    t0.record(stream)
    for k in range(steps):
        step(evs[k])
    t1.record(stream)
    torch.cuda.synchronize()
    if with_clocks is not None:
        with_clocks.__exit__(None, None, None)
    dg.sync()
    launch_ms = np.array([[a.elapsed_time(b) for (a, b) in row] for row in evs])
    return {"ms_total": t0.elapsed_time(t1), "launch_ms": launch_ms, "er": np.array(er, np.int64),
            "rr": np.array(rr, np.int64), "levels": np.array(lvls), "levels_buf": levels,
            "host_levels": host_levels}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="dfq", choices=["dfq", "reference"])
    ap.add_argument("--workload", default="rmat22", choices=["rmat22", "grid4096", "zipf262k", "batch", "serve"])
    ap.add_argument("--rates", default="1000,2000,5000,10000,20000,50000", help="serve: offered rates (q/s)")
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="serve: arrival window per rate")
    ap.add_argument("--serve-max", type=int, default=4000, help="serve: cap on requests per rate")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip the reference GPU kernel")
    ap.add_argument("--no-secondary", action="store_true", help="skip the 4096^2 grid secondary line")
    ap.add_argument("--sources", type=int, default=64)
    ap.add_argument("--scale", type=int, default=22,
                    help="R-MAT scale (22 is the benchmark; smaller scales are for profiler captures)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    ap.add_argument("--no-do", action="store_true", help="skip the direction-optimising line (reported separately)")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of every timed source")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-queries record")
    ap.add_argument("--ab", action="append", default=[], metavar="NAME=VALUE[,NAME=VALUE]",
                    help="option A/B: time the default options and each of these variants on the same "
                         "graph and sources (one JSON line), instead of the benchmark; repeatable")
    ap.add_argument("--pool-autotune", action="store_true",
                    help="batch workload: tune the batch kernel on the pool (dfq_pool_autotune) first")
    ap.add_argument("--level-profile", type=int, default=None, metavar="FROM",
                    help="per-level profile of the first source (64 levels from level FROM; with the "
                         "profiling build loaded through DFQ_LIB also the claim steps), one JSON line")
    ap.add_argument("--opt", action="append", default=[], metavar="NAME=VALUE",
                    help="kernel option for the timed graph (dfq_opts field), e.g. use_tma=0; repeatable")
    args = ap.parse_args()
    ws, rank, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        r = run_reference(args, ws, rank, pg)
        return r
    args.warmup = max(args.warmup, 3)

    import torch
    import dfqbfs as d
    torch.cuda.set_device(local)
    if args.workload == "batch":
        return run_batch(args, torch, d) if rank == 0 else 0
    if args.workload == "serve":
        return run_serve(args, torch, d) if rank == 0 else 0
    t_gen = time.perf_counter()
    g, all_srcs, cfg = workload_graph(args.workload, args.scale)
    t_gen = time.perf_counter() - t_gen
    srcs = all_srcs[: args.sources]
    o = kernel_opts(d, args)
    dg = d.Graph(g, opts=o)
    n = g.n
    if args.ab:
        return run_ab(args, dg, g, srcs, torch, d, cfg) if rank == 0 else 0
    if args.level_profile is not None:
        return run_level_profile(args, dg, g, srcs, torch, d, cfg) if rank == 0 else 0
    barrier(pg)
    ck = Clocks(local)
    m = measure_device(dg, srcs, n, args.steps, args.warmup, torch, with_clocks=ck,
                       keep_levels=(rank == 0 and not args.no_parity))
    barrier(pg)
    er, rr = m["er"], m["rr"]
    step_edges = int(er.sum())
    step_bytes = int((4 * er + 8 * rr + 4 * n).sum())
    ms_total = m["ms_total"]
    launch_ms = m["launch_ms"].ravel()
    levels = m["levels_buf"]
    ms_max = allreduce_max(pg, ms_total)
    total_edges = allreduce_sum(pg, float(step_edges * args.steps))
    value = total_edges / (ms_max * 1e-3) / 1e9
    hbm, peak_kind = peaks()
    avg_launch_ms = float(np.mean(launch_ms))
    bytes_per_launch = step_bytes / len(srcs)
    achieved = bytes_per_launch / (avg_launch_ms * 1e-3) / 1e9

    # e2e: public API with pinned host level buffers (launch + D2H inside the timed region)
    e2e, e2e_steps, ok_parity = None, 0, None
    if not args.no_e2e:
        host_lv = [torch.empty(n, dtype=torch.int32, pin_memory=True) for _ in range(2)]
        for i, s in enumerate(srcs[:4]):
            dg.bfs(int(s), levels_out=host_lv[i & 1])
        e2e_steps = max(1, min(args.steps, 3))
        barrier(pg)
        te0 = time.perf_counter()
        for _ in range(e2e_steps):
            for i, s in enumerate(srcs):
                dg.bfs(int(s), levels_out=host_lv[i & 1])
        te = time.perf_counter() - te0
        te = allreduce_max(pg, te)
        e2e_edges = allreduce_sum(pg, float(step_edges * e2e_steps))
        e2e = e2e_edges / te / 1e9
        # parity spot check of the e2e output against the device run
        ok_parity = bool(torch.equal(host_lv[(len(srcs) - 1) & 1], levels[(len(srcs) - 1) & 1].cpu()))

    traffic = None
    tp = ROOT / "profiles" / f"traffic_{args.workload}.txt"
    if tp.exists():
        for line in tp.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch="):
                traffic = float(line.split("=", 1)[1])

    metric = METRIC if args.workload == "rmat22" else f"BFS GTEPS ({cfg['workload']})"
    out = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
           "config": dict(cfg, sources=len(srcs), parallelism=f"replicas x{ws}"),
           "kernel_opts": dg.opts().as_dict(), "edges_per_step": step_edges, "gen_s": round(t_gen, 2),
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                        "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                        "kernel": "dfq_bfs_kernel", "bytes_alg_per_launch": bytes_per_launch,
                        "avg_launch_ms": avg_launch_ms},
           "e2e": ({"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * len(srcs),
                    "d2h_bytes_per_step": 4 * n * len(srcs), "api": "dfq_bfs (host levels)",
                    "steps": e2e_steps, "parity_vs_device": ok_parity} if e2e is not None else None),
           "gpu_launches": args.steps * len(srcs),
           "clocks": ck.summary(),
           "per_bfs_ms_median": float(np.median(launch_ms)),
           "us_per_level": float(np.median(m["launch_ms"][0] * 1e3 / np.maximum(m["levels"], 1)))}
    if cfg.get("symmetrized") or args.workload == "grid4096":
        # Graph500 counts an undirected edge once: E_R / 2 on a symmetrised graph
        out["graph500_gteps"] = value / 2
    if args.workload == "rmat22" and not args.no_do:
        out["direction_optimizing"] = direction_optimizing(g, srcs, er, rr, levels, args, torch, d, pg)
    if rank == 0 and not args.no_parity:
        # every timed source's levels (from the untimed pass) against the oracle
        out["parity"] = oracle_parity(g.offsets, g.cols, srcs, lambda i: m["host_levels"][i], device_er=er)
        m["host_levels"].clear()
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.lib()
        edges, tcpu, nsrc = cpu_sample(g, srcs, budget_s=15.0)
        out["cpu_baseline"] = {"value": edges / tcpu / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{nsrc} of the {len(srcs)} sources, serial oracle BFS, {tcpu:.1f} s",
                               "host": host_cpu()}
    if rank == 0 and not args.no_ref_gpu:
        import oracle
        k = 16 if args.workload == "rmat22" else 2
        wants = [oracle.bfs(g.offsets, g.cols, int(s)) for s in srcs[:k]]
        out["reference_gpu"] = reference_gpu(g, srcs, max_sources=k, wants=wants)
        # the global-queue baseline of the reference's design space, on the first 4 of them
        out["reference_gpu_global"] = reference_gpu(g, srcs, max_sources=min(4, k), kind="global", wants=wants)
    dg.close()
    if rank == 0 and args.workload == "rmat22" and not args.no_secondary:
        out["secondary"] = secondary_grid(torch, d, args)
    if rank == 0 and args.workload == "rmat22" and not args.no_batch:
        # the batch kernel tuned on the pool itself (dfq_pool_autotune, ~6 s), as a
        # user of the pool API would run it; the record keeps the default-option time too
        out["batch"] = batch_record(torch, d, min(args.steps, 3), 1, opts=kernel_opts(d, args), tune=True)
    if rank == 0:
        print(json.dumps(out))
    return 0


def run_ab(args, dg, g, srcs, torch, d, cfg):
    """Option A/B on one graph: the graph's options (defaults plus --opt) and
    each --ab variant, timed like the benchmark (events around every launch,
    `steps` passes over the sources after `warmup`), each variant's first
    source checked against the oracle.  One JSON line."""
    import oracle
    base = dg.opts()
    rows = []
    for spec in [""] + list(args.ab):
        o = d.Opts.from_buffer_copy(base)
        row = {"variant": spec or "base"}
        if spec == "autotune":  # dfq_autotune on the first 8 sources, from the defaults
            dg.set_opts(base)
            t0 = time.perf_counter()
            o = dg.autotune(srcs[:8])
            row["tune_s"] = round(time.perf_counter() - t0, 1)
            row["opts"] = o.as_dict()
        else:
            for kv in filter(None, spec.split(",")):
                k, v = kv.split("=", 1)
                setattr(o, k, int(v))
        try:
            dg.set_opts(o)
            m = measure_device(dg, srcs, g.n, args.steps, args.warmup, torch)
            lv = m["levels_buf"][(len(srcs) - 1) & 1].cpu().numpy()
            want = oracle.bfs(g.offsets, g.cols, int(srcs[-1]))
            row.update({"ms_per_bfs_mean": float(np.mean(m["launch_ms"])),
                        "ms_per_bfs_median": float(np.median(m["launch_ms"])),
                        "gteps": float(m["er"].sum() * m["launch_ms"].shape[0] / (m["launch_ms"].sum() * 1e-3) / 1e9),
                        "us_per_level": float(np.median(m["launch_ms"][0] * 1e3 / np.maximum(m["levels"], 1))),
                        "oracle_mismatches_last_source": int(oracle.compare(want, lv)["mismatches"])})
        except d.DfqError as e:
            row["error"] = str(e)
        rows.append(row)
    dg.set_opts(base)
    dg.close()
    print(json.dumps({"ab": rows, "config": dict(cfg, sources=len(srcs)), "steps": args.steps,
                      "warmup": args.warmup, "clock": "CUDA events around each launch"}))
    return 0


def run_level_profile(args, dg, g, srcs, torch, d, cfg):
    """Per-level profile (dfq_bfs_last_levels with profile on) of the first
    source after `warmup` runs: frontier, edges, the time to the last block's
    finish, the spread of block finishes, the barrier, the phase ends and - in
    the profiling build - the claim steps, for 64 levels from --level-profile."""
    o = dg.opts()
    o.profile = max(1, args.level_profile)
    dg.set_opts(o)
    lv = torch.empty(g.n, dtype=torch.int32, device="cuda")
    for _ in range(max(args.warmup, 1) + 1):
        dg.launch(int(srcs[0]), lv)
    dg.sync()
    rows = dg.last_levels(64)
    print(json.dumps({"level_profile": rows, "source": int(srcs[0]), "config": cfg,
                      "kernel_opts": dg.opts().as_dict(), "library": os.environ.get("DFQ_LIB", "product build")}))
    dg.close()
    return 0


def direction_optimizing(g, srcs, er, rr, td_levels, args, torch, d, pg):
    """The same sources with direction-optimising levels (dfq_opts.direction = 1,
    Beamer et al. 2012): reported beside the headline, which stays top-down like
    the reference.  GTEPS uses the same E_R per source (the fixed work model),
    so it is directly comparable; the levels of the last source are checked
    against the top-down run's."""
    o = d.default_opts()
    o.direction = 1
    with d.Graph(g, opts=o) as dg:
        m = measure_device(dg, srcs, g.n, max(1, min(args.steps, 5)), 3, torch)
        same = bool(torch.equal(m["levels_buf"][(len(srcs) - 1) & 1], td_levels[(len(srcs) - 1) & 1]))
        bu_levels = sum(1 for r in dg.last_levels(64) if r["probe"] == 2)
    ms = allreduce_max(pg, m["ms_total"])
    steps = m["launch_ms"].shape[0]
    edges = allreduce_sum(pg, float(er.sum() * steps))
    hbm, peak_kind = peaks()
    bytes_per_launch = float((4 * er + 8 * rr + 4 * g.n).sum()) / len(srcs)
    avg_ms = float(np.mean(m["launch_ms"]))
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
    return {"value": edges / (ms * 1e-3) / 1e9, "unit": UNIT, "per_bfs_ms_median": float(np.median(m["launch_ms"])),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "peak_kind": peak_kind, "bytes_alg_per_launch": bytes_per_launch, "avg_launch_ms": avg_ms,
                         "note": "the same fixed byte model as the headline (4 E_R + 8 |R| + 4 N); a bottom-up "
                                 "level reads fewer columns than E_R counts"},
            "steps": steps, "levels_match_top_down": same, "bottom_up_levels_last_source": bu_levels,
            "note": "same E_R per source as the headline; levels whose frontier holds > 1/14 of the "
                    "unexplored edges run bottom-up; not the reference's algorithm, so not the headline"}


def secondary_grid(torch, d, args):
    """The 4096^2 grid (high diameter): GTEPS and microseconds per level over its
    16 sources (4 corners, 12 interior), every source checked against the
    oracle, next to the reference kernel on one of them."""
    g, srcs, cfg = workload_graph("grid4096", 22)
    with d.Graph(g) as dg:
        m = measure_device(dg, srcs, g.n, 1, 1, torch, keep_levels=not args.no_parity)
    ms = m["launch_ms"][0]
    res = {"workload": cfg["workload"], "sources": srcs.tolist(), "gteps": float(m["er"].sum() / (ms.sum() * 1e-3) / 1e9),
           "ms_median": float(np.median(ms)), "levels_median": float(np.median(m["levels"])),
           "us_per_level": float(np.median(ms * 1e3 / np.maximum(m["levels"], 1)))}
    if not args.no_parity:
        res["parity"] = oracle_parity(g.offsets, g.cols, srcs, lambda i: m["host_levels"][i], device_er=m["er"])
        m["host_levels"].clear()
    if not args.no_ref_gpu:
        res["reference_gpu"] = reference_gpu(g, srcs[:1], max_sources=1)
    res["streams"] = streams_record(torch, d, args)
    return res


def streams_record(torch, d, args, side=1024, k=16, cluster=4, reps=3):
    """Throughput of many high-diameter searches at once through the
    single-graph API: k graph handles of the same side^2 grid (1 % of edges
    deleted, largest component), each with its own stream, all k searches
    launched (dfq_bfs_launch) before any is waited for (dfq_graph_sync).  The
    whole-GPU cooperative kernel runs them one after another; the cluster form
    (cluster_blocks = `cluster`, 1,024-thread blocks) runs them side by side.
    Host wall clock from the first launch to the last sync, best of `reps`;
    every result checked against the oracle."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    g, _ = d.gen_grid(side, 0.01, seed=1)
    srcs = [int(x) for x in g.pick_sources(k, seed=3)]
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        wants = list(ex.map(lambda s: oracle.bfs(g.offsets, g.cols, s), srcs))
    res = {"graph": f"grid {side}^2, 1% edges deleted, largest component", "n": int(g.n), "searches": k}
    for name, c in (("whole_gpu", 0), ("cluster", cluster)):
        o = d.default_opts()
        o.block_threads = 1024
        o.cluster_blocks = c
        hs = [d.Graph(g, opts=o) for _ in range(k)]
        try:
            lvs = [torch.empty(g.n, dtype=torch.int32, device="cuda") for _ in range(k)]
            best = float("inf")
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for h, s, lv in zip(hs, srcs, lvs):
                    h.launch(s, lv)
                for h in hs:
                    h.sync()
                best = min(best, time.perf_counter() - t0)
            bad = sum(oracle.compare(w, lv.cpu().numpy())["mismatches"] for w, lv in zip(wants, lvs))
        finally:
            for h in hs:
                h.close()
        res[name] = {"cluster_blocks": c, "ms_all": best * 1e3, "searches_per_s": k / best, "mismatches": int(bad)}
    res["speedup"] = res["cluster"]["searches_per_s"] / res["whole_gpu"]["searches_per_s"]
    return res


def reference_gpu(g, srcs, max_sources=16, kind="dfq", wants=None):
    """The reference kernel on the same graph: median GTEPS over sources.
    kind "dfq" = the shared-queue DFQ kernel, "global" = the global-queue
    baseline; wants = oracle levels of the sources, if already computed."""
    try:
        import oracle
        from oracle import refgpu
    except Exception as e:  # pragma: no cover
        return {"unavailable": f"import failed: {e}"}
    if not refgpu.available(kind):
        return {"unavailable": "reference cubin not built (reference sources absent where build() ran)"}
    kernels = {"dfq": "design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu",
               "global": "design/global-q/stripe-sa/gun-sep/lower-bound/bfs.cu"}
    res = {"kernel": kernels[kind], "sources": 0}
    try:
        with refgpu.RefGpu(kind) as ref:
            ref.load(g.offsets, g.cols)
            gteps, ms, errors = [], [], 0
            for i, s in enumerate(srcs[:max_sources]):
                want = wants[i] if wants is not None else oracle.bfs(g.offsets, g.cols, int(s))
                ok, why = ref.safe_for(want)
                if not ok:
                    return {"kernel": kernels[kind], "unavailable": f"refused (queue bounds): {why}"}
                ref.bfs(int(s))  # warm
                lv, t = ref.bfs(int(s))
                errors += oracle.compare(want, lv)["near_errors"]
                ms.append(t)
                gteps.append(oracle.reached_edges(g.offsets, want) / (t * 1e-3) / 1e9)
                depth = int(want.max())
            res.update({"sources": len(ms), "ms_median": float(np.median(ms)),
                        "us_per_level_last": float(ms[-1] * 1e3 / max(depth + 1, 1)),
                        "gteps_median": float(np.median(gteps)),
                        "gteps_aggregate": float(sum(g_ * m for g_, m in zip(gteps, ms)) / sum(ms)),
                        "errors": int(errors), "grid": ref.grid})
    except Exception as e:
        return {"kernel": kernels[kind], "unavailable": f"{type(e).__name__}: {e}"}
    return res


if __name__ == "__main__":
    sys.exit(main())
