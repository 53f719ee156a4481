"""Benchmark: the star query with bloom predicate transfer on one GB300.

Workload (the reference's SSB-SF1-shaped star query): fact 6,000,000 rows x
{fk1..fk4 int32, qty int32, price_cents int64, discount int32}, dims of
30,000 / 200,000 / 2,000 / 2,556 rows, dim filters keeping 1/5, 1/25, 1/7,
1/7, forward + backward blooms (10 bits/key, 3 hashes), 4-way hash join,
group by two dim attributes (~175 groups) with exact int64 sums. Seeded
synthetic data (SplitMix64), generated on the host.

A step is one execution of the physical plan (TableScan -> Filter ->
BloomFilterCreate / BloomFilterUse chains -> HashJoinArrow x4 -> Group ->
Collate) through the C ABI gfpdb_execute_plan, every kernel re-run on the
inputs each step.
  value : fact rows/s, inputs resident in HBM, the plan's operator pipeline
          captured once as a CUDA graph and replayed each step
          ("cudaGraph": true; deferred row counts, one synchronization).
  plain : the same plan launched operator by operator each step (the
          drop-in per-operator path), reported beside value.
  e2e   : the graph path with the tables in pinned host memory: every input's
          host-to-device copy and the result's device-to-host copy are inside
          the timed region.
The dominant kernel's roofline comes from a separate profiled pass of the
plain path on one stream (CUDA events around every launch).
With --gpus N (torchrun), each rank runs its own fact partition (weak
scaling, no collective on the data path); value = all ranks' fact rows / the
slowest rank's time.

--impl reference times the CPU restatement of the same query (oracle C port,
all host threads) on the same workload.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "fact rows/s & queries/s batched vs plain GPU path (bit-exact); p50/p99 latency"
UNIT = "fact rows/s"
FACT_ROWS = 6_000_000


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the benchmark runs."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples: list[list[str]] = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.1)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_baseline(tables, steps: int, warmup: int, budget_s: float):
    """The oracle's C restatement of the same query on the host cores."""
    from oracle import cbaseline

    inputs = cbaseline.StarInputs(tables)
    threads = os.cpu_count() or 1
    for _ in range(max(1, warmup)):
        cbaseline.star_query(inputs, threads=threads)
    times = []
    t_end = time.perf_counter() + budget_s
    while len(times) < steps or (time.perf_counter() < t_end and len(times) < 10_000):
        t0 = time.perf_counter()
        cbaseline.star_query(inputs, threads=threads)
        times.append(time.perf_counter() - t0)
    rows = tables["fact"].num_rows
    return {
        "value": rows * len(times) / sum(times),
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"full {rows}-row star query (bloom transfer + 4 joins + group-by), {len(times)} runs, "
                  f"{sum(times):.1f} s of wall time on {threads} threads",
        "ms_per_query": 1e3 * statistics.median(times),
    }


def run_reference(args, rank, world):
    from flexpushdowndb_gb300 import workloads

    if rank != 0:
        return
    tables = workloads.star_tables(fact_rows=FACT_ROWS, seed=2000)
    base = cpu_baseline(tables, args.steps, args.warmup, budget_s=args.cpu_seconds)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["ms_per_query"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic (SplitMix64-seeded)",
        "config": {"workload": "star query with bloom predicate transfer, fact 6,000,000 rows (SSB-SF1 shape)",
                   "fact_rows": FACT_ROWS, "host_threads": base["cores"]},
        "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _nth_newline(text: bytes, n: int) -> int:
    """Byte offset just past the n-th newline (the end of the first n rows)."""
    import numpy as np

    nl = np.flatnonzero(np.frombuffer(text, dtype=np.uint8) == 10)
    return int(nl[n - 1]) + 1


def _kernel_profile(L, _abi, fn, reps: int) -> dict:
    """Per-kernel event timings of `reps` calls of fn (profiling on)."""
    _abi.check(L.gfpdb_profile_reset())
    _abi.check(L.gfpdb_profile_enable(1))
    for _ in range(reps):
        fn()
    _abi.check(L.gfpdb_profile_enable(0))
    buf = ctypes.create_string_buffer(4096)
    _abi.check(L.gfpdb_profile_kernels(buf, 4096))
    out = {}
    for name in buf.value.decode().split():
        n, t_ms, by = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        _abi.check(L.gfpdb_profile_read(name.encode(), n, t_ms, by))
        out[name] = {"launches": n.value, "ms": t_ms.value, "bytes": by.value}
    return out


def batched_section(args, L, sptr, tabs) -> dict:
    """The batched form: the star query's fact table as 64 partitions of
    log-uniform size (59,952,713 rows), 32 query variants with dimension
    filter ranges of 1%-40% selectivity each. Batched: one gfpdb_star_batch
    call (one launch per stage for all partitions and queries, replayed as a
    CUDA graph). Plain: each query as its own physical plan (one scan per
    partition), launched operator by operator; per-query graph: the same
    plans captured and replayed one at a time. Every query's batched result
    is compared with its plain plan's."""
    from flexpushdowndb_gb300 import _abi, batch, plan, workloads
    from flexpushdowndb_gb300.tupleset import DeviceTable

    parts = [f"p{i}" for i in range(64)]
    qs = workloads.batch_queries(32)
    nq = len(qs)
    rows = sum(tabs[p].num_rows for p in parts)
    dev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
    spec = workloads.star_batch_spec(parts, qs)
    # items per thread, CTAs per SM and join-table load factor picked by
    # measurement (the tuner checks every candidate's results are identical)
    from flexpushdowndb_gb300 import autotune

    tuned = autotune.tune_star_batch(spec, dev, cache=None)
    spec = dict(spec, **tuned["settings"])
    for _ in range(args.warmup):
        batch.star_batch(spec, dev, stream=sptr)
    times = []
    for _ in range(max(args.steps, 10)):
        t0 = time.perf_counter()
        r = batch.star_batch(spec, dev, stream=sptr)
        times.append(time.perf_counter() - t0)
    got = batch.split_by_query(r.table)
    kern = _kernel_profile(L, _abi, lambda: batch.star_batch(spec, dev, use_graph=False, stream=sptr), 3)
    # plain per-query plans, operator by operator
    texts = [workloads.star_plan(ranges=q, fact_tables=parts).to_json() for q in qs]
    plan.execute(texts[0], dev, stream=sptr)
    parity = True
    plain = []
    for q in range(nq):
        t0 = time.perf_counter()
        res = plan.execute(texts[q], dev, stream=sptr)
        plain.append(time.perf_counter() - t0)
        parity &= res.table.sorted_rows() == got.get(q, [])
    # per-query graphs: a few queries, each captured then replayed
    graph = []
    for q in range(4):
        text = json.dumps(dict(json.loads(texts[q]), cudaGraph=True))
        for _ in range(2):
            plan.execute(text, dev, stream=sptr)
        for _ in range(5):
            t0 = time.perf_counter()
            plan.execute(text, dev, stream=sptr)
            graph.append(time.perf_counter() - t0)
        batch.clear_graph_cache()
    t_batch = statistics.median(times)
    t_plain = sum(plain) / len(plain)
    t_graph = statistics.median(graph)
    lat = sorted(times)
    fact = kern.get("sb_fact_kernel")
    return {
        "workload": "star query over 64 fact partitions (log-uniform 50,000-4,000,000 rows, %d in all), "
                    "32 variants with dimension filter ranges of 1%%-40%% selectivity" % rows,
        "fact_rows": rows, "queries": nq,
        "queries_per_s": nq / t_batch,
        "fact_rows_per_s": rows * nq / t_batch,
        "ms_per_batch": 1e3 * t_batch,
        "latency_ms": {"p50": 1e3 * lat[len(lat) // 2], "p99": 1e3 * lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "plain_per_query": {"queries_per_s": 1 / t_plain, "ms_per_query": 1e3 * t_plain},
        "graph_per_query": {"queries_per_s": 1 / t_graph, "ms_per_query": 1e3 * t_graph,
                            "note": "median over 4 of the 32 queries, each captured and replayed"},
        "speedup_vs_plain": t_plain * nq / t_batch,
        "speedup_vs_graph_per_query": t_graph * nq / t_batch,
        "parity_vs_plain": parity,
        "kernels_us_per_batch": {k: 1e3 * v["ms"] / 3 for k, v in kern.items()},
        "fact_kernel_fk_gbs": (fact["bytes"] / (fact["ms"] / 1e3) / 1e9) if fact else None,
        "settings": {k: spec[k] for k in ("itemsPerThread", "blocksPerSm", "loadFactor")},
        "autotune": {"ms_per_batch_default": tuned["default_ms"], "ms_per_batch_tuned": tuned["ms"],
                     "configurations_measured": tuned["measured"]},
    }


def csv_section(args, L, text: bytes, rows: int) -> dict:
    """The CSV form: 6,000,000 lineitem-shaped rows of '|'-delimited text
    (16 fields: 4 int32, 4 decimal(15,2), 2 dates, 6 strings of 10-40
    characters). Ingest: every field parsed into Arrow columns (int32, int64
    cents, date32, utf8) from device-resident text, timed by CUDA events
    around the parse kernels. Scan: the CsvScanPOp -> FilterPOp (three range
    predicates, ~2% selected) -> AggregatePOp (sum(d2 * i2), count) plan,
    from device-resident text and, end to end, from page-locked host text
    (the text's host-to-device copy inside the timed region). The CPU
    baseline parses the same text with the C restatement on every host
    thread."""
    from flexpushdowndb_gb300 import _abi, ops, plan, workloads
    from flexpushdowndb_gb300.tupleset import DeviceTable, export_host, text_table
    from oracle import cbaseline

    tt = text_table(text, "text")
    dev = DeviceTable.from_host(tt)
    text_ptr = dev.tensors[0][1].data_ptr()

    def ingest():
        return ops.csv_read(len(text), workloads.LINEITEM_FIELDS, delimiter="|", device_ptr=text_ptr, to_host=False)

    assert ingest() == rows
    kern = _kernel_profile(L, _abi, ingest, 3)
    csv_ms = sum(v["ms"] for v in kern.values()) / 3  # every kernel of the parse
    t_ingest = []
    for _ in range(5):
        t0 = time.perf_counter()
        ingest()
        t_ingest.append(time.perf_counter() - t0)
    scan_text = workloads.csv_scan_plan().to_json()
    dev_in = plan.PreparedInputs({"lineitem": dev})
    host_in = plan.PreparedInputs({"lineitem": export_host(tt, pinned=True)})
    got = plan.execute(scan_text, dev_in).table.rows()
    for _ in range(2):
        plan.execute(scan_text, dev_in)
    t_scan, t_e2e = [], []
    for _ in range(max(args.steps // 2, 5)):
        t0 = time.perf_counter()
        plan.execute(scan_text, dev_in)
        t_scan.append(time.perf_counter() - t0)
    plan.execute(scan_text, host_in)
    for _ in range(5):
        t0 = time.perf_counter()
        plan.execute(scan_text, host_in)
        t_e2e.append(time.perf_counter() - t0)
    threads = os.cpu_count() or 1
    cpu_t = []
    cpu = None
    t_end = time.perf_counter() + min(args.cpu_seconds, 10.0)
    while not cpu_t or (time.perf_counter() < t_end and len(cpu_t) < 20):
        t0 = time.perf_counter()
        cpu = cbaseline.csv_scan(text, workloads.CSV_T1_RANGE, workloads.CSV_D1_LT, workloads.CSV_I1_LT, threads)
        cpu_t.append(time.perf_counter() - t0)
    ti, ts, te, tc = (statistics.median(x) for x in (t_ingest, t_scan, t_e2e, cpu_t))
    return {
        "workload": "%d lineitem-shaped rows, %d bytes of '|'-delimited text (16 fields)" % (rows, len(text)),
        "ingest": {"rows_per_s": rows / (csv_ms / 1e3), "text_gbs": len(text) / (csv_ms / 1e3) / 1e9,
                   "kernel_ms": csv_ms, "call_ms": 1e3 * ti,
                   "kernels_ms": {k: v["ms"] / 3 for k, v in kern.items()}},
        "scan": {"rows_per_s": rows / ts, "ms": 1e3 * ts, "result": got},
        "scan_e2e": {"rows_per_s": rows / te, "ms": 1e3 * te, "h2d_bytes_per_step": len(text) + 8},
        "cpu_baseline": {"rows_per_s": rows / tc, "ms": 1e3 * tc, "cores": threads, "kind": "port",
                         "sample": f"the full {rows}-row scan, {len(cpu_t)} runs"},
        "parity_vs_cpu": got == [tuple(cpu)] if cpu[1] else got == [],
    }


def micro_section() -> dict:
    """Operator micro-benchmarks in the reference's shapes
    (fpdb-executor/bench/BloomFilterBenchmark.cpp:91-127,
    HashJoinBenchmark.cpp:99-131): tables of 10 int64 columns; bloom create
    over R rows with keys uniform on [0, 2R]; bloom use of R rows (keys
    uniform on [0, 2000]) against a filter of 10,000 keys uniform on
    [0, 1000]; hash join of L build x R probe rows on the first column (keys
    uniform on [0, 2R]) keeping three probe and two build columns. Device-resident inputs; median wall time per call
    of the C ABI (every call synchronizes its stream)."""
    import numpy as np

    from flexpushdowndb_gb300 import ops
    from flexpushdowndb_gb300.tupleset import Column, DeviceTable, Table

    rng = np.random.default_rng(11000)

    def table(rows, hi, prefix="c"):
        cols = [Column(f"{prefix}_0", "int64", rng.integers(0, hi + 1, rows))]
        cols += [Column(f"{prefix}_{i}", "int64", rng.integers(0, 1 << 40, rows)) for i in range(1, 10)]
        return DeviceTable.from_host(Table(cols))

    def med(fn, reps=20):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return 1e6 * statistics.median(ts)

    out = {"bloom_create_us": {}, "bloom_use_us": {}, "hash_join_us": {}}
    for r in (10, 100, 1000, 10_000, 100_000, 1_000_000):
        t = table(r, 2 * r)
        out["bloom_create_us"][str(r)] = med(lambda: ops.BloomFilter([t], "c_0"))
    bf = ops.BloomFilter([table(10_000, 1000)], "c_0")
    for r in (10, 100, 1000, 10_000, 100_000, 1_000_000):
        t = table(r, 2000)
        out["bloom_use_us"][str(r)] = med(lambda: bf.use(t, "c_0"))
    for left, right in ((10, 100), (10, 1000), (10, 10_000), (100, 1000), (100, 10_000), (1000, 10_000)):
        lt, rt = table(left, 2 * right, "b"), table(right, 2 * right)

        def join():
            j = ops.HashJoin("b_0", "c_0", ["c_0", "c_1", "c_2", "b_1", "b_2"])
            j.put_build(lt)
            j.finalize_build()
            return j.probe(rt)

        out["hash_join_us"][f"{left}x{right}"] = med(join)
    return out


def serving_section(args, batch_tabs, csv_text_2m) -> dict:
    """The serving form: Poisson arrivals of a request mix, swept over
    offered rates, through the request server (4 workers on their own
    streams, HBM column cache, admission by HBM budget, continuous batching
    of star queries, graphs) and through the plain path (one worker, every
    request its own per-operator plan, one stream, no batching). Latency is
    the server's finish - submit time. Templates: star queries with range
    filters over the 64-partition fact table (59,952,713 rows) and over its
    first 16 partitions; the two-table query and the star query with
    predicate transfer at 6,000,000 fact rows; the CSV scan over 2,000,000
    lineitem rows (484 MB of text, parsed per request); a group-by over
    20,000,000 rows with 10,000,000 Zipf(1.1) int64 keys."""
    import numpy as np

    from flexpushdowndb_gb300 import serving, workloads
    from flexpushdowndb_gb300.tupleset import text_table

    tables = dict(batch_tabs)
    two = workloads.two_table_tables(fact_rows=6_000_000, seed=1000)
    tables["fact"], tables["dim"] = two["fact"], two["dim"]
    star = workloads.star_tables(fact_rows=6_000_000, seed=2000)
    tables["sfact"] = star["fact"]
    for i in range(1, 5):
        tables[f"s{i}"] = star[f"d{i}"]
    tables["g"] = workloads.groupby_table(20_000_000, 10_000_000)
    tables["lineitem"] = text_table(csv_text_2m)
    from flexpushdowndb_gb300.tupleset import export_host

    tables = {k: export_host(v, pinned=True) for k, v in tables.items()}  # shared by every server below

    parts64 = [f"p{i}" for i in range(64)]
    parts16 = parts64[:16]
    tmpl = {64: serving.star_batch_template(workloads.star_batch_spec(parts64, [])),
            16: serving.star_batch_template(workloads.star_batch_spec(parts16, []))}
    star_plan = json.loads(workloads.star_plan().to_json())
    for o in star_plan["ops"]:
        if o["type"] == "TableScanPOp":
            o["table"] = "sfact" if o["table"] == "fact" else "s" + o["table"][1:]
    two_plan = json.loads(workloads.two_table_plan().to_json())
    csv_plan = json.loads(workloads.csv_scan_plan().to_json())
    g_plan = json.loads(workloads.groupby_plan(groups_hint=8_000_000).to_json())
    g_plan["ops"][0]["table"] = "g"
    rng = np.random.default_rng(7000)
    qranges = workloads.batch_queries(512, seed=7100)

    def request(k, plain):
        """The k-th request of the mix, as the served form or the plain form."""
        u = rng.random()
        if u < 0.72:  # star range query, 64 or 16 partitions
            n = 64 if u < 0.54 else 16
            q = qranges[k % len(qranges)]
            if plain:
                p = json.loads(workloads.star_plan(ranges=q, fact_tables=parts64 if n == 64 else parts16).to_json())
                return {"kind": "plan", "plan": p}
            return {"kind": "star", "batch": tmpl[n], "ranges": [list(r) for r in q]}
        if u < 0.82:
            return {"kind": "plan", "plan": two_plan}
        if u < 0.92:
            return {"kind": "plan", "plan": star_plan}
        if u < 0.96:
            return {"kind": "plan", "plan": csv_plan}
        return {"kind": "plan", "plan": g_plan}

    rates = [10, 100, 500, 1000, 2000, 4000, 8000]

    def sweep(plain):
        sv = serving.Server(workers=1 if plain else 4, batching=not plain, cuda_graphs=not plain,
                            plan_streams=1 if plain else 2, cache_bytes=100 << 30, hbm_budget_bytes=140 << 30)
        try:
            for name, t in tables.items():
                sv.register(name, t)
            # warm-up: every template once (loads the cache, prepares batches)
            rng.bit_generator.state = np.random.default_rng(7000).bit_generator.state
            warm = [request(k, plain) for k in range(40)]
            serving.run_load(sv, warm, [0.0] * len(warm))
            out = []
            for rate in rates:
                n = int(min(rate * args.serve_seconds, 4000 if not plain else 600))
                rng.bit_generator.state = np.random.default_rng(7000 + rate).bit_generator.state
                gaps = rng.exponential(1.0 / rate, n)
                arrivals = list(np.cumsum(gaps) - gaps[0])
                reqs = [request(k, plain) for k in range(n)]
                r = serving.run_load(sv, reqs, arrivals)
                out.append({"offered_qps": rate, "requests": n, "achieved_qps": r.achieved_qps,
                            "p50_ms": r.percentile(50), "p99_ms": r.percentile(99), "failed": r.failed,
                            "mean_batch": float(np.mean(r.batch_sizes)) if r.batch_sizes else 0.0})
                if r.achieved_qps < 0.6 * rate:
                    break  # saturated: higher rates only grow the queue
            st = sv.stats()
        finally:
            sv.close()
        return out, st

    def parity_check():
        """A sample of requests served both ways: identical results."""
        served_sv = serving.Server(workers=4, cache_bytes=100 << 30, hbm_budget_bytes=140 << 30)
        plain_sv = serving.Server(workers=1, batching=False, cuda_graphs=False, plan_streams=1,
                                  cache_bytes=100 << 30, hbm_budget_bytes=140 << 30)
        try:
            for name, t in tables.items():
                served_sv.register(name, t)
                plain_sv.register(name, t)
            ok = True
            for k in range(24):
                state = np.random.default_rng(9000 + k).bit_generator.state
                rng.bit_generator.state = state
                a = request(k, False)
                rng.bit_generator.state = state
                b = request(k, True)
                ta, tb = served_sv.submit(a), plain_sv.submit(b)
                ok &= served_sv.wait(ta)[0].sorted_rows() == plain_sv.wait(tb)[0].sorted_rows()
            return ok
        finally:
            served_sv.close()
            plain_sv.close()

    served, st_served = sweep(False)
    plain, _ = sweep(True)
    parity = parity_check()
    return {
        "workload": "Poisson arrivals; mix: 54% star range queries over 59,952,713 fact rows (64 partitions), "
                    "18% over 16 partitions, 10% two-table query (6M fact), 10% star query with bloom transfer "
                    "(6M fact), 4% CSV scan (2M lineitem rows of text, parsed per request), 4% group-by "
                    "(20M rows, 10M Zipf(1.1) int64 keys)",
        "served": served, "plain": plain, "parity_served_vs_plain": parity,
        "server": {"workers": 4, "cache_bytes": 100 << 30, "hbm_budget_bytes": 140 << 30,
                   "cache_hits": st_served["cache_hits"], "cache_misses": st_served["cache_misses"],
                   "batches": st_served["batches"], "batched_requests": st_served["batched_requests"],
                   "admission_waits": st_served["admission_waits"]},
        "plain_path": "1 worker, every request its own per-operator plan on one stream, no batching, no graphs",
    }


def run_case(args):
    """Single-kernel cases for profiling (ncu) and kernel tuning; prints one
    JSON line with the case's own timing. `select`: the forward bloom probe of
    the star query (fk2 against the 1/25 dim filter) over the 6M-row fact
    table, as one BloomFilterUsePOp runs it; `select4`: all four forward
    probes fused in one pass; `batch`: the batched star query (32 variants)
    over the first --parts partitions of the batched workload, stages launched
    without a graph."""
    import torch

    from flexpushdowndb_gb300 import ops, workloads
    from flexpushdowndb_gb300.expression import col, eq, num_lit
    from flexpushdowndb_gb300.tupleset import DeviceTable
    from oracle import ops as oops

    ops.init(0)
    if args.case == "batch":
        from flexpushdowndb_gb300 import batch, plan

        tabs = workloads.batch_tables(args.parts)
        parts = [f"p{i}" for i in range(args.parts)]
        dev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
        spec = workloads.star_batch_spec(parts, workloads.batch_queries(32))
        fn = lambda: batch.star_batch(spec, dev, use_graph=False).table  # noqa: E731
        args.rows = sum(tabs[p].num_rows for p in parts)
        return _time_case(args, fn)
    if args.case in ("join", "group", "csv", "filter"):
        return _operator_case(args)
    tabs = workloads.star_tables(fact_rows=args.rows, seed=2000)
    fact = DeviceTable.from_host(tabs["fact"])
    if args.case == "plan-timeline":
        return _plan_timeline(args, tabs)
    if args.case in ("plan", "plan-graph"):
        from flexpushdowndb_gb300 import plan

        d = json.loads(workloads.star_plan().to_json())
        if args.case == "plan-graph":
            d["cudaGraph"] = True
        text = json.dumps(d)
        inputs = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
        fn = lambda: plan.execute(text, inputs).table  # noqa: E731
    elif args.case == "select":
        d2 = oops.filter_table(tabs["d2"], eq(col("d2_f"), num_lit(3)))
        bf = ops.BloomFilter([d2], "d2_pk")
        fn = lambda: ops.select(fact, blooms=[(bf, "fk2")])  # noqa: E731
    elif args.case == "select4":
        blooms = []
        for i, c in ((2, 3), (3, 2), (4, 5), (1, 1)):
            d = oops.filter_table(tabs[f"d{i}"], eq(col(f"d{i}_f"), num_lit(c)))
            blooms.append((ops.BloomFilter([d], f"d{i}_pk"), f"fk{i}"))
        fn = lambda: ops.select(fact, blooms=blooms)  # noqa: E731
    else:
        raise SystemExit(f"unknown case {args.case}")
    return _time_case(args, fn)


def _operator_case(args):
    """Single operators at sizes past the L2, for their ncu captures:
    `join`: args.rows probe rows (int32 keys uniform over the build keys and
    10% more, two payload columns) against args.rows / 10 unique build keys,
    fixed-width outputs (one probe-and-materialise kernel); `group`: args.rows
    rows of Zipf(1.1) int64 keys over args.rows / 2 keys, sum and count;
    `csv`: the lineitem text of args.rows rows parsed on the device;
    `filter`: a two-comparison range conjunction (~2% of rows) over an int32
    and an int64 column of args.rows rows, projecting an int32 and an int64
    column; prints the kernel's algorithmic GB/s beside the call time."""
    import numpy as np

    from flexpushdowndb_gb300 import ops, workloads
    from flexpushdowndb_gb300.expression import col
    from flexpushdowndb_gb300.tupleset import Column, DeviceTable, Table

    ops.init(0)
    n = args.rows
    rng = np.random.default_rng(7000)
    if args.case == "join":
        nb = max(1, n // 10)
        build = Table([Column("pk", "int32", rng.permutation(nb)), Column("bv", "int64", rng.integers(0, 10**9, nb))])
        probe = DeviceTable.from_host(Table([Column("fk", "int32", rng.integers(0, nb + nb // 10, n)),
                                             Column("pv", "int32", rng.integers(0, 100, n))]))
        j = ops.HashJoin("pk", "fk")
        j.put_build(DeviceTable.from_host(build))
        j.finalize_build()
        fn = lambda: j.probe(probe)  # noqa: E731
        for _ in range(max(2, args.warmup)):
            fn()
        # the probe and the output rows: the fused probe-and-materialise
        # kernel, or the pair probe and its gather
        ms = _kernel_ms(fn, ("join_probe_kernel", "join_probe_emit_kernel", "gather_fixed_kernel"), args.steps)
        print(json.dumps({"case": "join", "rows": n, "build_rows": nb, "probe_and_output_ms": ms,
                          "probes_per_s": n / (ms * 1e-3)}))
    elif args.case == "group":
        t = DeviceTable.from_host(workloads.groupby_table(n, max(1, n // 2)))
        aggs = [ops.aggregate("SUM", "s", col("v")), ops.aggregate("COUNT", "c")]

        def fn():
            g = ops.Group(["k"], aggs)
            g.group(t)
            return g.finalise()

        for _ in range(max(2, args.warmup)):
            fn()
        from flexpushdowndb_gb300 import _abi

        prof = _kernel_profile(_abi.lib(), _abi, fn, args.steps)
        print(json.dumps({"case": "group", "rows": n, "kernels_ms": {k: v["ms"] / args.steps for k, v in prof.items()}}))
    elif args.case == "filter":
        from flexpushdowndb_gb300.expression import and_, gte, lt, num_lit

        t = Table([Column("a", "int32", rng.integers(0, 1000, n)), Column("b", "int64", rng.integers(0, 10**9, n)),
                   Column("c", "int32", rng.integers(0, 100, n)), Column("d", "int64", rng.integers(0, 10**12, n))])
        dt = DeviceTable.from_host(t)
        pred = and_(lt(col("a"), num_lit(100)), gte(col("b"), num_lit(800_000_000, "int64")))
        f = ops.Filter(pred, t)
        fn = lambda: f.evaluate(dt, project=["c", "d"])  # noqa: E731
        out = fn()
        sel = out.num_rows
        for _ in range(max(3, args.warmup)):
            fn()
        ms = _kernel_ms(lambda: f.evaluate(dt, project=["c", "d"]),
                        ("select_kernel", "select_probe_kernel", "select_gather_kernel"), args.steps)
        algo = n * 12 + sel * 24  # a, b over every row; c, d read and written for the selected rows
        print(json.dumps({"case": "filter", "rows": n, "selected": sel, "kernel_ms": ms,
                          "algorithmic_gbs": algo / (ms * 1e6)}))
        return
    else:
        import torch

        text = workloads.lineitem_csv(n)
        dev = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda()

        class _Rows:
            def __init__(self, k):
                self.num_rows = k

        fn = lambda: _Rows(ops.csv_read(len(text), workloads.LINEITEM_FIELDS, delimiter="|",  # noqa: E731
                                        device_ptr=dev.data_ptr(), to_host=False))
    return _time_case(args, fn)


def _kernel_ms(fn, names, reps):
    """Mean device time (CUDA events around each launch) of the named
    kernels per call of fn."""
    from flexpushdowndb_gb300 import _abi

    prof = _kernel_profile(_abi.lib(), _abi, fn, reps)
    return sum(v["ms"] for k, v in prof.items() if k in names) / reps


def _plan_timeline(args, tabs):
    """Kernel timeline of one replay of the captured star plan (CUPTI kernel
    records through torch.profiler): per kernel its start and end relative
    to the replay's first kernel and its duration. Prints one JSON line per
    kernel, then a summary line."""
    import torch
    from torch.profiler import ProfilerActivity, profile

    from flexpushdowndb_gb300 import plan, workloads
    from flexpushdowndb_gb300.tupleset import DeviceTable

    d = json.loads(workloads.star_plan().to_json())
    d.update({"cudaGraph": True, "streams": args.streams})
    pp = plan.PreparedPlan(json.dumps(d), plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()}))
    for _ in range(max(3, args.warmup)):
        pp.execute()
    torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CUDA]):  # the first session of a process records nothing
        torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        for _ in range(3):
            r = pp.execute()
        torch.cuda.synchronize()
    evs = [e for e in prof.events() if e.device_type == torch.autograd.DeviceType.CUDA]
    evs.sort(key=lambda e: e.time_range.start)
    # the last replay: kernels after the last gap of more than 20 us
    steps, cur = [], []
    for e in evs:
        if cur and e.time_range.start - max(x.time_range.end for x in cur) > 20:
            steps.append(cur)
            cur = []
        cur.append(e)
    steps.append(cur)
    last = steps[-1]
    t0 = last[0].time_range.start
    for e in last:
        name = e.name.replace("(anonymous namespace)::", "").replace("gfpdb::", "").replace("void ", "")
        print(json.dumps({"kernel": name.split("(")[0].split("<")[0],
                          "start_us": round(e.time_range.start - t0, 1), "end_us": round(e.time_range.end - t0, 1),
                          "us": round(e.time_range.end - e.time_range.start, 1)}))
    print(json.dumps({"case": "plan-timeline", "streams": args.streams, "kernels": len(last),
                      "span_us": round(max(e.time_range.end for e in last) - t0, 1),
                      "device_ms_reported": r.stats["device_ns"] / 1e6}))


def _time_case(args, fn):
    import torch

    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = fn()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.steps
    print(json.dumps({"case": args.case, "rows": args.rows, "ms_per_call": 1e3 * dt, "rows_out": out.num_rows}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gfpdb", choices=["gfpdb", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--case", default=None, help="profiling case: select | select4 | plan | plan-graph | plan-timeline | batch | join | group | csv")
    ap.add_argument("--parts", type=int, default=64, help="fact partitions of the batch case")
    ap.add_argument("--rows", type=int, default=FACT_ROWS)
    ap.add_argument("--streams", type=int, default=4, help="plan streams for --case plan-timeline")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-form section")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-form section")
    ap.add_argument("--no-csv", action="store_true", help="skip the CSV-form section")
    ap.add_argument("--no-micro", action="store_true", help="skip the operator micro-benchmarks")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival window per offered rate")
    args = ap.parse_args()
    if args.case:
        return run_case(args)
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world if "RANK" in os.environ else 1)

    import torch

    dist = None
    if "RANK" in os.environ and world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    from flexpushdowndb_gb300 import _abi, ops, plan, workloads
    from flexpushdowndb_gb300.tupleset import DeviceTable
    from oracle import queries

    torch.cuda.set_device(local)
    ops.init(local)
    L = _abi.lib()
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    tables = workloads.star_tables(fact_rows=FACT_ROWS, seed=2000 + 7 * rank)
    plan_d = json.loads(workloads.star_plan().to_json())
    plain_text = json.dumps(plan_d)
    graph_text = json.dumps(dict(plan_d, cudaGraph=True))
    dev_inputs = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tables.items()})
    host_inputs = plan.PreparedInputs(tables, pinned=True)
    input_bytes = sum(t.nbytes() for t in tables.values())
    want = queries.star_query(tables).sorted_rows()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def timed(text, inputs, steps):
        """K steps bracketed by barrier + synchronize; CUDA events on the
        stream for the region and for each step."""
        prepared = plan.PreparedPlan(text, inputs, stream=sptr)
        events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        per = []
        stats = None
        device_ms, call_ms = [], []
        ev0.record(stream)
        for a, b in events:
            a.record(stream)
            r = prepared.execute()
            b.record(stream)
            per.append((a, b))
            stats = r.stats
            device_ms.append(r.stats.get("device_ns", 0) / 1e6)
            call_ms.append(r.stats.get("elapsed_ns", 0) / 1e6)
        ev1.record(stream)
        barrier()
        timed.device_ms = device_ms
        timed.call_ms = call_ms
        return ev0.elapsed_time(ev1) / steps, [a.elapsed_time(b) for a, b in per], stats, r

    def timed_pipelined(text, inputs, steps):
        """K steps through two prepared instances of the plan (graph
        instances 0 and 1, each with its own capture and result buffers)
        launched alternately on the stream: step k is launched, then step
        k - 1 is waited for and its result read on the host while step k runs,
        so the GPU does not idle through the host's turnaround. Bracketed by
        barrier + synchronize and CUDA events like timed()."""
        d = json.loads(text)
        preps = [plan.PreparedPlan(json.dumps(dict(d, graphInstance=i)), inputs, stream=sptr) for i in (0, 1)]
        for pp in preps:
            for _ in range(3):  # the ordinary run, the capture, a replay
                pp.execute()
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        preps[0].launch()
        for k in range(1, steps):
            preps[k % 2].launch()
            r = preps[(k - 1) % 2].wait()
        r = preps[(steps - 1) % 2].wait()
        ev1.record(stream)
        barrier()
        return ev0.elapsed_time(ev1) / steps, r

    def e2e_pipelined(text, inputs, steps):
        """Wall time per step of K steps through two prepared instances on
        two streams, launched alternately (each waited for while the other
        runs)."""
        d = json.loads(text)
        sts = [torch.cuda.Stream() for _ in range(2)]
        preps = [plan.PreparedPlan(json.dumps(dict(d, graphInstance=i)), inputs, stream=sts[i].cuda_stream)
                 for i in (0, 1)]
        for pp in preps:
            for _ in range(3):
                pp.execute()
        barrier()
        t0 = time.perf_counter()
        preps[0].launch()
        for k in range(1, steps):
            preps[k % 2].launch()
            r = preps[(k - 1) % 2].wait()
        r = preps[(steps - 1) % 2].wait()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
        barrier()
        return dt, r

    with ClockSampler(local) as clocks:
        # parity of every path (outside the timed regions), bit-exact
        parity = all(plan.execute(t, i, stream=sptr).table.sorted_rows() == want
                     for t, i in ((plain_text, dev_inputs), (graph_text, dev_inputs), (graph_text, dev_inputs),
                                  (graph_text, host_inputs), (graph_text, host_inputs)))
        # ---- value: captured plan, device-resident inputs
        for _ in range(args.warmup):
            plan.execute(graph_text, dev_inputs, stream=sptr)
        launches0 = ops.kernel_launches()
        ms, per_step, _, last = timed(graph_text, dev_inputs, args.steps)
        graph_device_ms = statistics.median(timed.device_ms)
        graph_call_ms = statistics.median(timed.call_ms)
        launches = (ops.kernel_launches() - launches0) / args.steps
        parity = parity and last.table.sorted_rows() == want
        seq_ms = max_over_ranks(ms)
        # value: the same replays, two prepared instances launched back to back
        ms, last = timed_pipelined(graph_text, dev_inputs, args.steps)
        parity = parity and last.table.sorted_rows() == want
        ms = max_over_ranks(ms)
        value = FACT_ROWS * world / (ms / 1e3)
        # ---- plain per-operator path, same inputs
        for _ in range(args.warmup):
            plan.execute(plain_text, dev_inputs, stream=sptr)
        plain_ms, plain_steps, _, _ = timed(plain_text, dev_inputs, args.steps)
        plain_ms = max_over_ranks(plain_ms)
        # ---- e2e: pinned host inputs through the same C-ABI call; the scans
        # copy them with the copy engine or with SM loads over the
        # chip-to-chip link, and the faster of the two is reported
        e2e_modes, e2e_pipe = {}, {}
        for mode in ("engine", "sm", "zerocopy"):
            text = json.dumps(dict(plan_d, cudaGraph=True, hostCopy=mode))
            parity = parity and plan.execute(text, host_inputs, stream=sptr).table.sorted_rows() == want
            for _ in range(args.warmup):
                plan.execute(text, host_inputs, stream=sptr)
            barrier()
            e2e_times = []
            prepared = plan.PreparedPlan(text, host_inputs, stream=sptr)
            for _ in range(args.steps):
                t0 = time.perf_counter()
                r = prepared.execute()
                torch.cuda.synchronize()
                e2e_times.append(time.perf_counter() - t0)
            barrier()
            e2e_modes[mode] = (max_over_ranks(sum(e2e_times) / len(e2e_times)), r.stats)
            if mode != "zerocopy":
                # two prepared instances on two streams, launched alternately:
                # each step still copies all its inputs in and reads its
                # result, while the other step's kernels run
                pipe_s, r = e2e_pipelined(text, host_inputs, args.steps)
                parity = parity and r.table.sorted_rows() == want
                e2e_pipe[mode] = (max_over_ranks(pipe_s), r.stats)
        # e2e counts only paths that copy every input across; the zero-copy
        # scan (kernels read host columns in place) is reported beside it
        e2e_mode = min(("engine", "sm"), key=lambda m: e2e_pipe[m][0])
        e2e_s, e2e_stats = e2e_pipe[e2e_mode]
        h2d, d2h = e2e_stats["h2d_bytes"], e2e_stats["d2h_bytes"]
        # ---- profiled pass: every kernel launch of the plain path timed with
        # CUDA events on its stream, algorithmic bytes per launch
        _abi.check(L.gfpdb_profile_reset())
        _abi.check(L.gfpdb_profile_enable(1))
        # one stream here: event timings of kernels that overlap on several
        # streams would count the overlap twice
        timed(json.dumps(dict(plan_d, streams=1)), dev_inputs, args.steps)
        _abi.check(L.gfpdb_profile_enable(0))

    buf = ctypes.create_string_buffer(4096)
    _abi.check(L.gfpdb_profile_kernels(buf, 4096))
    kernels = {}
    for name in buf.value.decode().split():
        n, t_ms, by = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        _abi.check(L.gfpdb_profile_read(name.encode(), n, t_ms, by))
        kernels[name] = {"launches": n.value, "ms": t_ms.value, "bytes": by.value}
    gpu_ms_total = sum(k["ms"] for k in kernels.values())
    top = max(kernels, key=lambda k: kernels[k]["ms"]) if kernels else None
    peak, peak_kind = _peaks()
    traffic_by = {}
    tp = ROOT / "profiles" / "traffic.txt"
    if tp.exists():
        for ln in tp.read_text().splitlines():
            f = ln.split()
            if len(f) == 2 and not ln.startswith("#"):
                traffic_by[f[0]] = float(f[1])

    def roofline_of(name):
        # achieved = algorithmic bytes per launch / mean event-timed launch
        # duration; traffic = ncu DRAM bytes per launch of the same kernel
        k = kernels[name]
        achieved = k["bytes"] / (k["ms"] / 1e3) / 1e9
        launches = max(1, k["launches"])
        return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "traffic": traffic_by.get(name), "launches_per_step": k["launches"] / args.steps,
                "avg_launch_us": 1e3 * k["ms"] / launches,
                "algorithmic_bytes_per_launch": k["bytes"] / launches,
                "share_of_kernel_time": k["ms"] / gpu_ms_total if gpu_ms_total else None}

    roofline = roofline_of(top) if top else None
    # the largest-input kernel (the fact-table scan) beside the top-by-time one
    fact_scan = "select_probe_kernel" if "select_probe_kernel" in kernels else None
    roofline_fact = roofline_of(fact_scan) if fact_scan else None

    # the batched form runs after the timed region, on every rank (replicas)
    # the autotuner on the star plan (bloom bits / hashes, join load factor,
    # streams); the headline keeps the workload's 10 bits/key, 3 hashes
    from flexpushdowndb_gb300 import autotune

    autotune_plan = autotune.tune_star_plan(plan_d, dev_inputs, cache=None)
    batch_tabs = None if (args.no_batched and args.no_serving) else workloads.batch_tables()
    batched = None if args.no_batched else batched_section(args, L, sptr, batch_tabs)
    csv_text = None if (args.no_csv and args.no_serving) else workloads.lineitem_csv(
        6_000_000, processes=os.cpu_count() or 1)
    csv = None if args.no_csv else csv_section(args, L, csv_text, 6_000_000)
    micro = None if args.no_micro else micro_section()
    # the serving form's CSV template reads the first 2,000,000 rows
    cut = None if csv_text is None else _nth_newline(csv_text, 2_000_000)
    serving = None if args.no_serving else serving_section(args, batch_tabs, csv_text[:cut])

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    base = None
    if world == 1 and not args.no_cpu_baseline:
        b = cpu_baseline(tables, 3, 1, budget_s=args.cpu_seconds)
        base = {k: b[k] for k in ("value", "unit", "cores", "kind", "sample")}
        # the same C port on one thread (SURVEY: "1 thread and all cores")
        from oracle import cbaseline

        inp = cbaseline.StarInputs(tables)
        t0 = time.perf_counter()
        cbaseline.star_query(inp, threads=1)
        base["one_thread_value"] = FACT_ROWS / (time.perf_counter() - t0)
    lat = sorted(per_step)
    plat = sorted(plain_steps)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "graph_device_ms": graph_device_ms,
        "graph_library_call_ms": graph_call_ms,
        "sequential": {"value": FACT_ROWS * world / (seq_ms / 1e3), "ms_per_step": seq_ms,
                       "note": "one prepared plan, each step launched after the previous one's result was read"},
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic (SplitMix64-seeded), generated on the host",
        "config": {"workload": "star query with bloom predicate transfer, fact 6,000,000 rows (SSB-SF1 shape)",
                   "fact_rows_per_gpu": FACT_ROWS, "dims": [30000, 200000, 2000, 2556],
                   "bloom": "10 bits/key, 3 hashes, forward + backward",
                   "path": "plan captured as a CUDA graph (deferred row counts), replayed per step; two prepared "
                           "instances launched back to back, each step's result read on the host",
                   "l2": "inputs (%.0f MB) larger than the 129 MB L2; no flush needed" % (input_bytes / 1e6),
                   "parallelism": f"replicas x{world}"},
        "queries_per_s": world * 1e3 / ms,
        # per-step latency of the sequential run (one query at a time)
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "plain": {"value": FACT_ROWS * world / (plain_ms / 1e3), "ms_per_step": plain_ms,
                  "queries_per_s": world * 1e3 / plain_ms,
                  "latency_ms": {"p50": plat[len(plat) // 2], "p99": plat[min(len(plat) - 1, int(0.99 * len(plat)))]}},
        "parity": parity,
        "e2e": {"value": FACT_ROWS * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s, "host_copy": e2e_mode,
                "pipeline": "two prepared instances on two streams, launched alternately",
                "ms_per_step_by_copy": {m: 1e3 * v[0] for m, v in e2e_pipe.items()},
                "sequential_ms_per_step_by_copy": {m: 1e3 * v[0] for m, v in e2e_modes.items()}},
        "e2e_zero_copy": {"value": FACT_ROWS * world / e2e_modes["zerocopy"][0], "unit": UNIT,
                          "note": "host columns read in place over NVLink-C2C by the scan kernels; "
                                  "only touched sectors cross the link",
                          "ms_per_step": 1e3 * e2e_modes["zerocopy"][0]},
        "gpu_launches": launches,
        "roofline": roofline,
        "roofline_fact_scan": roofline_fact,
        "kernels": {k: {"launches_per_step": v["launches"] / args.steps, "us_per_step": 1e3 * v["ms"] / args.steps}
                    for k, v in kernels.items()},
        "clocks": clocks.summary(),
        "cpu_baseline": base,
        "autotune_star_plan": autotune_plan,
        "csv": csv,
        "micro": micro,
        "batched": batched,
        "serving": serving,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
