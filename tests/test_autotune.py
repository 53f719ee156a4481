"""The autotuner: coordinate descent and the settings cache (CPU), and tuning
the batched engine and the star plan on the GPU with exact results."""

import json

import pytest

from flexpushdowndb_gb300 import autotune


def test_coordinate_descent_finds_separable_minimum():
    space = {"a": [1, 2, 3, 4], "b": [10, 20, 30]}
    cost = lambda c: (c["a"] - 3) ** 2 + (c["b"] - 10) ** 2 / 100.0  # noqa: E731
    best, t, measured = autotune.coordinate_descent(space, {"a": 1, "b": 30}, cost)
    assert best == {"a": 3, "b": 10} and t == 0
    assert len(measured) <= 4 * 3


def test_cache_roundtrip(tmp_path):
    p = tmp_path / "tune.json"
    autotune._store(p, "k1", {"settings": {"x": 1}})
    autotune._store(p, "k2", {"settings": {"x": 2}})
    assert autotune._load(p)["k1"]["settings"] == {"x": 1}
    assert autotune._load(tmp_path / "missing.json") == {}


def test_apply_plan_settings():
    from flexpushdowndb_gb300 import workloads

    d = json.loads(workloads.star_plan().to_json())
    out = autotune.apply_plan_settings(d, {"bitsPerKey": 12, "numHashes": 2, "joinLoadFactor": 0.7, "streams": 2})
    assert out["streams"] == 2
    assert all(o["bitsPerKey"] == 12 and o["numHashes"] == 2 for o in out["ops"] if o["type"] == "BloomFilterCreatePOp")
    assert all(o["loadFactor"] == 0.7 for o in out["ops"] if o["type"] == "HashJoinArrowPOp")
    assert "streams" not in d  # the input plan is not modified


@pytest.mark.gpu
def test_tune_star_batch_and_plan(gpu, tmp_path):
    from flexpushdowndb_gb300 import plan, workloads
    from flexpushdowndb_gb300.tupleset import DeviceTable

    sizes = workloads.batch_partition_sizes(4, lo=5_000, hi=200_000, seed=8000)
    tabs = workloads.batch_tables(4, sizes=sizes, seed=8000)
    parts = [f"p{i}" for i in range(4)]
    dev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
    spec = workloads.star_batch_spec(parts, workloads.batch_queries(8, seed=8001))
    cache = tmp_path / "tune.json"
    space = {"itemsPerThread": [1, 2], "blocksPerSm": [2, 4], "loadFactor": [0.5, 0.7]}
    r = autotune.tune_star_batch(spec, dev, reps=2, cache=cache, space=space)
    assert r["settings"]["itemsPerThread"] in (1, 2) and r["ms"] <= r["default_ms"]
    assert autotune.tune_star_batch(spec, dev, cache=cache, space=space)["cached"]
    star = workloads.star_tables(fact_rows=200_000, seed=8002)
    sdev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in star.items()})
    pspace = {"bitsPerKey": [8, 10], "numHashes": [3], "joinLoadFactor": [0.5], "streams": [1, 4]}
    pr = autotune.tune_star_plan(json.loads(workloads.star_plan().to_json()), sdev, reps=3, cache=cache,
                                 space=pspace)
    assert pr["settings"]["bitsPerKey"] in (8, 10) and pr["ms"] <= pr["default_ms"]
