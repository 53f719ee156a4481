"""Bloom filters tested in the hash join build (pipeline fusion folds a
bloom selection that feeds only an inner join's build side into the join):
fused and unfused plans give the oracle's join, single joins and chains,
exact and device-sized filters, with and without graph capture; a join that
keeps unmatched build rows applies its build filters by a selection first."""

import json

import numpy as np
import pytest

from flexpushdowndb_gb300 import plan, workloads
from flexpushdowndb_gb300.expression import col, lt, num_lit
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops
from oracle import queries

pytestmark = pytest.mark.gpu


def tables(n_dim, n_fact, key_type, dup, seed):
    rng = np.random.default_rng(seed)
    keys = np.arange(1, n_dim + 1)
    if dup:
        keys = np.concatenate([keys, keys[: n_dim // 3]])
    dim = Table([Column("d_pk", key_type, keys), Column("d_v", "int64", rng.integers(-(2**40), 2**40, len(keys)))])
    # the fact references a tenth of the dimension: the backward filter
    # rejects most dimension rows
    fk = rng.integers(1, n_dim // 10 + 2, n_fact)
    fact = Table([Column("fk", key_type, fk), Column("x", "int32", rng.integers(0, 100, n_fact))])
    return {"dim": dim, "fact": fact}


def two_table(fact_filter, join_type="INNER", fuse=True, graph=False):
    p = plan.Plan()
    p.scan("scan_d", "dim", ["d_pk", "d_v"])
    p.scan("scan_f", "fact", ["fk", "x"])
    src = "scan_f"
    if fact_filter:  # a selection before the filter: its size is only known on the device
        src = p.filter("filter_f", "scan_f", lt(col("x"), num_lit(37, "int32")), ["fk", "x"])
    c = p.bloom_create("bw_create", src, "fk")
    u = p.bloom_use("bw_use", "scan_d", c, "d_pk")
    p.hash_join("join", u, c, "d_pk", "fk", ["x", "d_v"])
    p.op("join")["joinType"] = join_type
    p.collate("collate", "join")
    d = json.loads(p.to_json())
    d["fusePipelines"] = fuse
    if graph:
        d["cudaGraph"] = True
    return json.dumps(d)


def sort_rows(t):
    return sorted(t.rows(), key=lambda r: tuple((v is None, 0 if v is None else v) for v in r))


@pytest.mark.parametrize("key_type", ["int32", "int64"])
@pytest.mark.parametrize("dup", [False, True])
@pytest.mark.parametrize("fact_filter", [False, True])
@pytest.mark.parametrize("graph", [False, True])
def test_single_join_build_filter(gpu, key_type, dup, fact_filter, graph):
    tabs = tables(50_000, 300_000, key_type, dup, seed=7 + dup)
    fact = tabs["fact"]
    if fact_filter:
        keep = fact["x"] < 37
        fact = Table([Column(c.name, c.type, c.values[keep]) for c in fact.columns])
    want = oops.hash_join(tabs["dim"], fact, "d_pk", "fk", ["x", "d_v"]).sorted_rows()
    for fuse in (True, False):
        text = two_table(fact_filter, fuse=fuse, graph=graph)
        for _ in range(2 if graph else 1):
            r = plan.execute(text, tabs)
            assert r.table.names == ["x", "d_v"]
            assert r.table.sorted_rows() == want
        assert r.stats["num_ops"] == (5 if fuse else 6) + (1 if fact_filter else 0)


@pytest.mark.parametrize("jt", ["INNER", "LEFT", "RIGHT", "FULL", "LEFT_SEMI", "RIGHT_SEMI"])
def test_build_filters_any_join_type(gpu, jt):
    """A plan that carries "buildFilters" on a join of any type gives the
    rows of the same plan with the bloom selection before the join: joins
    that keep or mark build rows select first, inner and probe-side joins
    test the filter in the build."""
    tabs = tables(20_000, 100_000, "int32", True, seed=3)
    unfused = two_table(False, jt, fuse=False)
    want = plan.execute(unfused, tabs).table
    folded = plan.fused(two_table(False, "INNER"))
    for o in folded["ops"]:
        if o["name"] == "join":
            o["joinType"] = jt
    assert "buildFilters" in [o for o in folded["ops"] if o["name"] == "join"][0]
    folded["fusePipelines"] = False  # run exactly these operators
    got = plan.execute(json.dumps(folded), tabs).table
    assert got.names == want.names
    assert sort_rows(got) == sort_rows(want)
    # and the unfused plan is the oracle's typed join of the selected build side
    if jt in ("INNER", "RIGHT", "RIGHT_SEMI"):
        assert sort_rows(got) == sort_rows(
            oops.hash_join_typed(tabs["dim"], tabs["fact"], "d_pk", "fk", jt, ["x", "d_v"]))


@pytest.mark.parametrize("planned", [False, True])
def test_star_build_filters_match_oracle(gpu, planned):
    tabs = workloads.star_tables(fact_rows=500_000, seed=41)
    p = workloads.star_plan_planned(fact_rows=500_000) if planned else workloads.star_plan()
    want = queries.star_query(tabs).sorted_rows()
    fused = plan.fused(p)
    assert sum(1 for o in fused["ops"] if o["type"] == "BloomFilterUsePOp") == 1
    r = plan.execute(p, tabs)
    assert r.table.sorted_rows() == want
    assert r.stats["num_ops"] == 18


def two_filter_plan(fuse):
    """A dimension filtered by two fact tables' keys (two bloom uses in a
    chain, fused into one use with two probes, folded into the join build
    as two build filters); the join probes the first fact table."""
    p = plan.Plan()
    p.scan("scan_d", "dim", ["d_pk", "d_v"])
    p.scan("scan_f", "fact", ["fk", "x"])
    p.scan("scan_g", "fact2", ["gk"])
    c1 = p.bloom_create("bw1", "scan_f", "fk")
    c2 = p.bloom_create("bw2", "scan_g", "gk", 6, 2)
    u1 = p.bloom_use("use1", "scan_d", c1, "d_pk")
    u2 = p.bloom_use("use2", u1, c2, "d_pk")
    p.hash_join("join", u2, c1, "d_pk", "fk", ["x", "d_v"])
    p.collate("collate", "join")
    d = json.loads(p.to_json())
    d["fusePipelines"] = fuse
    return json.dumps(d)


@pytest.mark.parametrize("key_type", ["int32", "int64"])
def test_join_build_with_two_filters(gpu, key_type):
    tabs = tables(40_000, 200_000, key_type, True, seed=23)
    rng = np.random.default_rng(5)
    gk = rng.integers(1, 40_000, 3000)
    tabs["fact2"] = Table([Column("gk", key_type, gk)])
    fused = plan.fused(two_filter_plan(True))
    join = [o for o in fused["ops"] if o["name"] == "join"][0]
    assert [f["creator"] for f in join["buildFilters"]] == ["bw1", "bw2"]
    # the second filter keeps the dimension rows the oracle's filter over
    # fact2's keys keeps, false positives included; the first cannot drop a
    # row the join would emit
    keep = oops.bloom_contains(oops.bloom_words(tabs["fact2"]["gk"], 6, 2), tabs["dim"]["d_pk"], 2)
    dim = Table([Column(c.name, c.type, c.values[keep]) for c in tabs["dim"].columns])
    want = oops.hash_join(dim, tabs["fact"], "d_pk", "fk", ["x", "d_v"]).sorted_rows()
    for fuse in (True, False):
        r = plan.execute(two_filter_plan(fuse), tabs)
        assert r.table.sorted_rows() == want
