"""Autotuner for the launch and table parameters of the hot path.

Picks, by measurement on the current GPU:
  - the batched star engine's items per thread, CTAs per SM, foreign-key
    pipeline stages and join-table load factor (tune_star_batch);
  - a star plan's bloom bits per key and hash count, hash-join load factor and
    number of streams (tune_star_plan).
Search is coordinate descent from the defaults: one parameter at a time over
its candidates, keeping the best, until a full pass changes nothing. Every
candidate's result must equal the default configuration's result exactly (a
setting that changed a result would be a bug, and the tuner refuses it).
Choices are kept in a JSON file keyed by device and workload shape, so a
later process reuses them without measuring again.
"""

from __future__ import annotations

import json
import os
import statistics
import time
from pathlib import Path

from . import _abi, batch, plan

DEFAULT_CACHE = Path(os.environ.get("GFPDB_AUTOTUNE_CACHE", Path.home() / ".cache" / "gfpdb" / "autotune.json"))

BATCH_SPACE = {
    "itemsPerThread": [2, 4, 8],
    "blocksPerSm": [1, 2, 3, 4],
    "stages": [2, 3, 4, 6],
    "loadFactor": [0.3, 0.5, 0.7],
}

PLAN_SPACE = {
    "bitsPerKey": [6, 8, 10, 12, 16],
    "numHashes": [2, 3, 4],
    "joinLoadFactor": [0.3, 0.5, 0.7],
    "streams": [1, 2, 4, 8],
}


def device_name() -> str:
    import torch

    return torch.cuda.get_device_name(0) if torch.cuda.is_available() else "cpu"


def _load(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def _store(path: Path, key: str, value: dict) -> None:
    data = _load(path)
    data[key] = value
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
    tmp.replace(path)


def _time(fn, reps: int) -> float:
    fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def coordinate_descent(space: dict, start: dict, measure, max_passes: int = 3):
    """Minimise measure(config) one coordinate at a time. Returns (best
    config, its time, every (config, time) measured)."""
    best = dict(start)
    best_t = measure(best)
    seen = {json.dumps(best, sort_keys=True): best_t}
    for _ in range(max_passes):
        changed = False
        for name, values in space.items():
            for v in values:
                cand = dict(best, **{name: v})
                k = json.dumps(cand, sort_keys=True)
                if k not in seen:
                    seen[k] = measure(cand)
                if seen[k] < best_t:
                    best, best_t, changed = cand, seen[k], True
        if not changed:
            break
    return best, best_t, [(json.loads(k), t) for k, t in seen.items()]


def tune_star_batch(spec: dict, inputs, reps: int = 5, cache: Path | None = DEFAULT_CACHE, key: str | None = None,
                    space: dict = BATCH_SPACE) -> dict:
    """Tunes gfpdb_star_batch for `spec` (its queries included) over `inputs`
    (a PreparedInputs of device tables). Returns {"settings", "ms", "default_ms",
    "measured"}; the settings are cached under `key` (default: the device and
    the spec's partition count and query count)."""
    key = key or f"star_batch|{device_name()}|parts={len(spec['factTables'])}|queries={len(spec['queries'])}"
    if cache is not None:
        hit = _load(cache).get(key)
        if hit:
            return dict(hit, cached=True)
    start = {k: spec.get(k, BATCH_SPACE[k][1]) for k in space}
    want = batch.split_by_query(batch.star_batch(dict(spec, **start), inputs).table)

    def measure(cfg):
        s = dict(spec, **cfg)
        got = batch.split_by_query(batch.star_batch(s, inputs).table)
        if got != want:
            raise RuntimeError(f"tuning candidate {cfg} changed a result")
        t = _time(lambda: batch.star_batch(s, inputs), reps)
        batch.clear_graph_cache()  # each candidate's prepared batch and graph
        return t

    best, t, measured = coordinate_descent(space, start, measure)
    default_t = [x for c, x in measured if c == start][0]
    out = {"settings": best, "ms": 1e3 * t, "default_ms": 1e3 * default_t, "measured": len(measured)}
    if cache is not None:
        _store(cache, key, out)
    return out


def apply_plan_settings(plan_json: dict, settings: dict) -> dict:
    """The plan with the given bloom / join / stream settings."""
    d = json.loads(json.dumps(plan_json))
    for o in d["ops"]:
        if o["type"] == "BloomFilterCreatePOp":
            o["bitsPerKey"] = settings["bitsPerKey"]
            o["numHashes"] = settings["numHashes"]
        elif o["type"] == "HashJoinArrowPOp":
            o["loadFactor"] = settings["joinLoadFactor"]
    d["streams"] = settings["streams"]
    return d


def tune_star_plan(plan_json: dict, inputs, reps: int = 9, cache: Path | None = DEFAULT_CACHE,
                   key: str | None = None, space: dict = PLAN_SPACE) -> dict:
    """Tunes a star plan (graph-replayed) over `inputs`. Returns {"settings",
    "ms", "default_ms", "measured"}."""
    key = key or f"star_plan|{device_name()}|ops={len(plan_json['ops'])}"
    if cache is not None:
        hit = _load(cache).get(key)
        if hit:
            return dict(hit, cached=True)
    start = {"bitsPerKey": 10, "numHashes": 3, "joinLoadFactor": 0.5, "streams": 4}
    base = apply_plan_settings(plan_json, start)
    want = plan.execute(json.dumps(base), inputs).table.sorted_rows()

    def measure(cfg):
        text = json.dumps(dict(apply_plan_settings(plan_json, cfg), cudaGraph=True))
        if plan.execute(text, inputs).table.sorted_rows() != want:
            raise RuntimeError(f"tuning candidate {cfg} changed a result")
        t = _time(lambda: plan.execute(text, inputs), reps)
        _abi.check(_abi.lib().gfpdb_graph_cache_clear())
        return t

    best, t, measured = coordinate_descent(space, start, measure)
    default_t = [x for c, x in measured if c == start][0]
    out = {"settings": best, "ms": 1e3 * t, "default_ms": 1e3 * default_t, "measured": len(measured)}
    if cache is not None:
        _store(cache, key, out)
    return out
