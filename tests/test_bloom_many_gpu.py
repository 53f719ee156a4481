"""Several bloom filters over the same rows built in one pass
(bloom_build_many, behind BloomFilterCreatePOps that pipeline fusion
merges: a chain of creators forwarding the rows, or sibling creators on one
producer): each filter keeps exactly the rows the oracle's filter of the same
keys, bits per key and hash count keeps, false positives included, with exact
and device-sized inputs, fused and unfused."""

import json

import numpy as np
import pytest

from flexpushdowndb_gb300 import plan
from flexpushdowndb_gb300.expression import col, lt, num_lit
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops

pytestmark = pytest.mark.gpu

FILTERS = [("k1", "x1", 10, 3), ("k2", "x2", 7, 2), ("k1", "x3", 16, 4)]  # key, probe column, bits, hashes


def tables(n, m, seed):
    rng = np.random.default_rng(seed)
    t = Table([Column("k1", "int32", rng.integers(0, 1 << 30, n)), Column("k2", "int64", rng.integers(-(2**50), 2**50, n)),
               Column("v", "int32", rng.integers(0, 100, n))])
    # probe rows: a third hit the filter's keys, the rest are random (false positives)
    x = []
    for key, _, _, _ in FILTERS:
        pool = t[key]
        hit = pool[rng.integers(0, max(1, n), m)] if n else np.zeros(m, dtype=np.int64)
        miss = rng.integers(0, 1 << 30, m) if key == "k1" else rng.integers(-(2**50), 2**50, m)
        x.append(np.where(rng.random(m) < 1 / 3, hit, miss))
    xt = Table([Column("x1", "int32", x[0]), Column("x2", "int64", x[1]), Column("x3", "int32", x[2]),
                Column("id", "int64", np.arange(m))])
    return {"t": t, "x": xt}


def bloom_plan(shape, selective, fuse):
    p = plan.Plan()
    p.scan("scan_t", "t", ["k1", "k2", "v"])
    src = "scan_t"
    if selective:  # a device-sized input
        src = p.filter("filter_t", "scan_t", lt(col("v"), num_lit(40, "int32")), ["k1", "k2", "v"])
    creators = []
    prev = src
    for i, (key, _, bits, hashes) in enumerate(FILTERS):
        c = p.bloom_create(f"c{i}", prev if shape == "chain" else src, key, bits, hashes)
        creators.append(c)
        if shape == "chain":
            prev = c
    p.scan("scan_x", "x", ["x1", "x2", "x3", "id"])
    tail = "scan_x"
    for i, (_, xcol, _, _) in enumerate(FILTERS):
        tail = p.bloom_use(f"u{i}", tail, creators[i], xcol)
    p.collate("collate", tail)
    d = json.loads(p.to_json())
    d["fusePipelines"] = fuse
    return json.dumps(d)


@pytest.mark.parametrize("shape", ["chain", "siblings"])
@pytest.mark.parametrize("selective", [False, True])
@pytest.mark.parametrize("n", [0, 1, 3000, 400_000])
def test_filters_built_together_match_oracle(gpu, shape, selective, n):
    tabs = tables(n, 60_000, seed=n + (shape == "chain"))
    t = tabs["t"]
    keys = t
    if selective:
        keep = t["v"] < 40
        keys = Table([Column(c.name, c.type, c.values[keep]) for c in t.columns])
    ok = np.ones(tabs["x"].num_rows, dtype=bool)
    for key, xcol, bits, hashes in FILTERS:
        words = oops.bloom_words(keys[key], bits, hashes)
        ok &= oops.bloom_contains(words, tabs["x"][xcol], hashes)
    want = sorted(tabs["x"]["id"][ok].tolist())
    for fuse in (True, False):
        text = bloom_plan(shape, selective, fuse)
        if fuse:
            fused = plan.fused(text)
            merged = [o for o in fused["ops"] if o["type"] == "BloomFilterCreatePOp"]
            assert len(merged) == 1 and len(merged[0]["filters"]) == 3
        r = plan.execute(text, tabs)
        assert sorted(r.table["id"].tolist()) == want
