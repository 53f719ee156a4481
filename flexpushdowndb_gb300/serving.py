"""The request server (gfpdb_server_* in include/gfpdb.h) and a load driver.

Server wraps one native server: registered host tables, an HBM column cache,
worker threads on their own CUDA streams, admission by HBM budget and
continuous batching of star queries. run_load replays a request stream at
given arrival times (Poisson arrivals in the benchmark) and reports each
request's latency from the server's own clock.
"""

from __future__ import annotations

import ctypes
import json
import threading
import time
from dataclasses import dataclass

from . import _abi
from .tupleset import Exported, Table, export_host, import_result, new_output


class Server:
    def __init__(self, workers: int = 4, cache_bytes: int = 100 << 30, hbm_budget_bytes: int = 120 << 30,
                 max_batch: int = 64, batching: bool = True, plan_streams: int = 2, cuda_graphs: bool = True,
                 device: int = 0, admission_timeout_ms: int = 120_000):
        cfg = {"device": device, "workers": workers, "cacheBytes": cache_bytes, "hbmBudgetBytes": hbm_budget_bytes,
               "maxBatch": max_batch, "batching": batching, "planStreams": plan_streams, "cudaGraphs": cuda_graphs,
               "admissionTimeoutMs": admission_timeout_ms}
        self._h = ctypes.c_void_p()
        _abi.check(_abi.lib().gfpdb_server_create(json.dumps(cfg).encode(), ctypes.byref(self._h)))
        self._keep = []  # exported host tables: their buffers must outlive the server

    def register(self, name: str, table, pinned: bool = True) -> None:
        """Register a host Table (exported here, page-locked unless pinned is
        False) or an already exported one (tupleset.export_host), which
        several servers may share."""
        ex = table if isinstance(table, Exported) else export_host(table, pinned=pinned)
        self._keep.append(ex)
        _abi.check(_abi.lib().gfpdb_server_register_table(self._h, name.encode(), ex.schema_ptr, ex.array_ptr))

    def submit(self, request: dict | str) -> int:
        t = ctypes.c_uint64()
        text = request if isinstance(request, str) else json.dumps(request)
        _abi.check(_abi.lib().gfpdb_server_submit(self._h, text.encode(), ctypes.byref(t)))
        return t.value

    def submit_plan(self, plan) -> int:
        d = json.loads(plan.to_json()) if hasattr(plan, "to_json") else (json.loads(plan) if isinstance(plan, str) else plan)
        return self.submit({"kind": "plan", "plan": d})

    def submit_star(self, batch_template: dict, ranges) -> int:
        return self.submit({"kind": "star", "batch": batch_template, "ranges": [list(r) for r in ranges]})

    def wait(self, ticket: int, timeout_ms: int = -1, result: bool = True):
        """(Table or None, stats dict). Raises GfpdbError for a failed request,
        TimeoutError when it is not finished within timeout_ms."""
        st = _abi.RequestStats()
        if result:
            s, a = new_output()
            code = _abi.lib().gfpdb_server_wait(self._h, ticket, timeout_ms, ctypes.byref(s), ctypes.byref(a),
                                                 ctypes.byref(st))
        else:
            code = _abi.lib().gfpdb_server_wait(self._h, ticket, timeout_ms, None, None, ctypes.byref(st))
        if code == _abi.GFPDB_ETIMEDOUT and st.end_ns == 0:
            raise TimeoutError(f"request {ticket} not finished within {timeout_ms} ms")
        _abi.check(code)
        stats = {k: getattr(st, k) for k, _ in _abi.RequestStats._fields_ if k != "pad"}
        return (import_result(s, a) if result else None), stats

    def stats(self) -> dict:
        out = _abi.ServerStats()
        _abi.check(_abi.lib().gfpdb_server_get_stats(self._h, ctypes.byref(out)))
        return {k: getattr(out, k) for k, _ in _abi.ServerStats._fields_}

    def close(self) -> None:
        if self._h:
            _abi.check(_abi.lib().gfpdb_server_destroy(self._h))
            self._h = ctypes.c_void_p()
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def star_batch_template(spec: dict) -> dict:
    """A gfpdb_star_batch spec without its queries: the "batch" of a star request."""
    return {k: v for k, v in spec.items() if k != "queries"}


@dataclass
class LoadResult:
    offered_qps: float
    achieved_qps: float
    latencies_ms: list
    batch_sizes: list
    failed: int
    wall_s: float

    def percentile(self, p: float) -> float:
        if not self.latencies_ms:
            return float("nan")
        s = sorted(self.latencies_ms)
        return s[min(len(s) - 1, int(p / 100.0 * len(s)))]


def run_load(server: Server, requests: list, arrivals_s: list, timeout_ms: int = 300_000) -> LoadResult:
    """Submit requests[i] at arrivals_s[i] seconds after the start (open loop)
    and collect them all; latency = the server's finish - submit time."""
    tickets = [None] * len(requests)
    done = threading.Event()
    out = {"lat": [], "bs": [], "failed": 0}

    def collect():
        for i in range(len(requests)):
            while tickets[i] is None:
                time.sleep(0.0002)
            try:
                _, st = server.wait(tickets[i], timeout_ms, result=False)
                out["lat"].append((st["end_ns"] - st["submit_ns"]) / 1e6)
                out["bs"].append(st["batch_size"])
            except Exception:
                out["failed"] += 1
        done.set()

    th = threading.Thread(target=collect, daemon=True)
    th.start()
    t0 = time.perf_counter()
    for i, (req, at) in enumerate(zip(requests, arrivals_s)):
        delay = at - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        tickets[i] = server.submit(req)
    done.wait()
    wall = time.perf_counter() - t0
    n = len(requests)
    span = arrivals_s[-1] if arrivals_s and arrivals_s[-1] > 0 else 1.0
    return LoadResult(offered_qps=n / span, achieved_qps=(n - out["failed"]) / wall, latencies_ms=out["lat"],
                      batch_sizes=out["bs"], failed=out["failed"], wall_s=wall)
