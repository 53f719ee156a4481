"""Benchmark: the star query with bloom predicate transfer on one GB300.

Workload (the reference's SSB-SF1-shaped star query): fact 6,000,000 rows x
{fk1..fk4 int32, qty int32, price_cents int64, discount int32}, dims of
30,000 / 200,000 / 2,000 / 2,556 rows, dim filters keeping 1/5, 1/25, 1/7,
1/7, forward + backward blooms (10 bits/key, 3 hashes), 4-way hash join,
group by two dim attributes (~175 groups) with exact int64 sums. Seeded
synthetic data (SplitMix64), generated on the host.

A step is one execution of the physical plan (TableScan -> Filter ->
BloomFilterCreate / BloomFilterUse chains -> HashJoinArrow x4 -> Group ->
Collate) through the C ABI gfpdb_execute_plan.
  value : fact rows/s with every input table already resident in HBM.
  e2e   : the same call with the tables in pinned host memory; the
          host-to-device copies of every input and the device-to-host copy of
          the result are inside the timed region.
With --gpus N (torchrun), each rank runs its own fact partition (weak
scaling, no collective on the data path); value = all ranks' fact rows / the
slowest rank's time.

--impl reference times the CPU restatement of the same query (oracle C port,
all host threads) on the same workload.
"""

from __future__ import annotations

import argparse
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
    """nvidia-smi clock / throttle sampling during the timed region."""

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
            self._stop.wait(0.2)

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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gfpdb", choices=["gfpdb", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world if "RANK" in os.environ else 1)

    import numpy as np
    import torch

    dist = None
    if "RANK" in os.environ and world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    from flexpushdowndb_gb300 import _abi, ops, plan, workloads
    from flexpushdowndb_gb300.tupleset import DeviceTable

    torch.cuda.set_device(local)
    ops.init(local)
    L = _abi.lib()
    stream = torch.cuda.current_stream()
    sptr = ctypes_stream(stream)

    tables = workloads.star_tables(fact_rows=FACT_ROWS, seed=2000 + 7 * rank)
    star = workloads.star_plan()
    text = star.to_json()
    dev_inputs = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tables.items()})
    host_inputs = plan.PreparedInputs(tables, pinned=True)
    input_bytes = sum(t.nbytes() for t in tables.values())

    # parity check (outside the timed region): bit-exact against the oracle
    from oracle import queries

    got = plan.execute(text, dev_inputs, stream=sptr).table
    want = queries.star_query(tables)
    parity = got.sorted_rows() == want.sorted_rows()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- value: device-resident inputs
    for _ in range(args.warmup):
        plan.execute(text, dev_inputs, stream=sptr)
    _abi.check(L.gfpdb_profile_reset())
    _abi.check(L.gfpdb_profile_enable(1))
    launches0 = ops.kernel_launches()
    step_ms = []
    with ClockSampler(local) as clocks:
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            plan.execute(text, dev_inputs, stream=sptr)
            b.record(stream)
            step_ms.append((a, b))
        ev1.record(stream)
        barrier()
    _abi.check(L.gfpdb_profile_enable(0))
    launches = (ops.kernel_launches() - launches0) / args.steps
    total_ms = ev0.elapsed_time(ev1)
    per_step = [a.elapsed_time(b) for a, b in step_ms]
    ms = total_ms / args.steps
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = FACT_ROWS * world / (ms / 1e3)

    # per-kernel live timings from the timed region
    buf = ctypes_buffer(4096)
    _abi.check(L.gfpdb_profile_kernels(buf, 4096))
    kernels = {}
    for name in buf.value.decode().split():
        n, t_ms, by = ctypes_i64(), ctypes_f64(), ctypes_f64()
        _abi.check(L.gfpdb_profile_read(name.encode(), n, t_ms, by))
        kernels[name] = {"launches": n.value, "ms": t_ms.value, "bytes": by.value}
    gpu_ms_total = sum(k["ms"] for k in kernels.values())
    top = max(kernels, key=lambda k: kernels[k]["ms"]) if kernels else None
    peak, peak_kind = _peaks()
    roofline = None
    if top:
        k = kernels[top]
        achieved = k["bytes"] / (k["ms"] / 1e3) / 1e9
        traffic = None
        tp = ROOT / "profiles" / "traffic.json"
        if tp.exists():
            traffic = json.loads(tp.read_text()).get(top)
        roofline = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                    if peak_kind == "measured" else "fallback 6.8 TB/s",
                    "traffic": traffic, "launches_per_step": k["launches"] / args.steps,
                    "avg_launch_us": 1e3 * k["ms"] / max(1, k["launches"]),
                    "algorithmic_bytes_per_launch": k["bytes"] / max(1, k["launches"]),
                    "share_of_kernel_time": k["ms"] / gpu_ms_total if gpu_ms_total else None}

    # ---- e2e: pinned host inputs, copies inside the timed region
    for _ in range(args.warmup):
        plan.execute(text, host_inputs, stream=sptr)
    barrier()
    e2e_times = []
    h2d = d2h = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = plan.execute(text, host_inputs, stream=sptr)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
        h2d, d2h = r.stats["h2d_bytes"], r.stats["d2h_bytes"]
    barrier()
    e2e_s = sum(e2e_times) / len(e2e_times)
    if dist is not None:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    if rank != 0:
        dist.destroy_process_group() if dist is not None else None
        return
    base = None
    if world == 1 and not args.no_cpu_baseline:
        b = cpu_baseline(tables, 3, 1, budget_s=args.cpu_seconds)
        base = {k: b[k] for k in ("value", "unit", "cores", "kind", "sample")}
    lat = sorted(per_step)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic (SplitMix64-seeded), generated on the host",
        "config": {"workload": "star query with bloom predicate transfer, fact 6,000,000 rows (SSB-SF1 shape)",
                   "fact_rows_per_gpu": FACT_ROWS, "dims": [30000, 200000, 2000, 2556],
                   "bloom": "10 bits/key, 3 hashes, forward + backward", "path": "plain per-operator plan",
                   "l2": "inputs (%.0f MB) larger than the 129 MB L2" % (input_bytes / 1e6),
                   "parallelism": f"replicas x{world}"},
        "queries_per_s": world * 1e3 / ms,
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "parity": parity,
        "e2e": {"value": FACT_ROWS * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s},
        "gpu_launches": launches,
        "roofline": roofline,
        "kernels": {k: {"launches_per_step": v["launches"] / args.steps, "us_per_step": 1e3 * v["ms"] / args.steps}
                    for k, v in kernels.items()},
        "clocks": clocks.summary(),
        "cpu_baseline": base,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def ctypes_stream(stream):
    import ctypes

    return ctypes.c_void_p(stream.cuda_stream)


def ctypes_buffer(n):
    import ctypes

    return ctypes.create_string_buffer(n)


def ctypes_i64():
    import ctypes

    return ctypes.c_int64()


def ctypes_f64():
    import ctypes

    return ctypes.c_double()


if __name__ == "__main__":
    main()
