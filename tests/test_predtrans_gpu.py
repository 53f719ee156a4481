"""Plans whose bloom predicate transfer the planner derived from the join
graph (Plan.predicate_transfer) give the oracle's results: the star query,
and a four-table snowflake chain where filters travel two joins."""

import numpy as np
import pytest

from flexpushdowndb_gb300 import ops, plan, workloads
from flexpushdowndb_gb300.expression import col, eq, lte, num_lit
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops
from oracle import queries

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ranges", [None, [(0, 30), (0, 10), (3, 50), (0, 99)]])
def test_planned_star_query(gpu, ranges):
    tabs = workloads.star_tables(fact_rows=400_000, seed=77)
    got = plan.execute(workloads.star_plan_planned(fact_rows=400_000, ranges=ranges), tabs).table
    if ranges is None:
        want = queries.star_query(tabs)
    else:
        want = queries.star_query_ranges({**tabs, "p0": tabs["fact"]}, ["p0"], ranges)
    assert got.sorted_rows() == want.sorted_rows()


def snowflake(seed=5):
    rng = np.random.default_rng(seed)
    region = Table([Column("r_regionkey", "int32", np.arange(5)), Column("r_code", "int32", np.arange(5) * 10)])
    nation = Table([Column("n_nationkey", "int32", np.arange(25)), Column("n_regionkey", "int32", np.arange(25) % 5)])
    ns = 2000
    supplier = Table([Column("s_suppkey", "int32", np.arange(ns)),
                      Column("s_nationkey", "int32", rng.integers(0, 25, ns))])
    nl = 200_000
    lineitem = Table([Column("l_suppkey", "int32", rng.integers(0, ns, nl)),
                      Column("l_price", "int64", rng.integers(100, 10_000, nl))])
    return {"region": region, "nation": nation, "supplier": supplier, "lineitem": lineitem}


@pytest.mark.parametrize("code", [20, 40])
def test_planned_snowflake_chain(gpu, code):
    t = snowflake()
    p = plan.Plan()
    p.scan("scan_region", "region")
    p.filter("filter_region", "scan_region", eq(col("r_code"), num_lit(code)), ["r_regionkey"])
    for name in ("nation", "supplier", "lineitem"):
        p.scan(f"scan_{name}", name)
    out = p.predicate_transfer(
        {"filter_region": (5, 0.2), "scan_nation": 25, "scan_supplier": 2000, "scan_lineitem": 200_000},
        [{"left": "scan_nation", "right": "filter_region", "leftColumns": ["n_regionkey"], "rightColumns": ["r_regionkey"]},
         {"left": "scan_supplier", "right": "scan_nation", "leftColumns": ["s_nationkey"], "rightColumns": ["n_nationkey"]},
         {"left": "scan_lineitem", "right": "scan_supplier", "leftColumns": ["l_suppkey"], "rightColumns": ["s_suppkey"]}])
    j1 = p.hash_join("j_rn", out["filter_region"], out["scan_nation"], "r_regionkey", "n_regionkey", ["n_nationkey"])
    j2 = p.hash_join("j_ns", j1, out["scan_supplier"], "n_nationkey", "s_nationkey", ["s_suppkey", "s_nationkey"])
    j3 = p.hash_join("j_sl", j2, out["scan_lineitem"], "s_suppkey", "l_suppkey", ["s_nationkey", "l_price"])
    p.group("g", j3, ["s_nationkey"], [ops.aggregate("SUM", "rev", col("l_price")), ops.aggregate("COUNT", "n")])
    p.collate("collate", "g")
    plan.validate(p)
    got = plan.execute(p, t).table

    r = oops.filter_table(t["region"], eq(col("r_code"), num_lit(code)), ["r_regionkey"])
    rn = oops.hash_join(r, t["nation"], "r_regionkey", "n_regionkey", ["n_nationkey"])
    ns = oops.hash_join(rn, t["supplier"], "n_nationkey", "s_nationkey", ["s_suppkey", "s_nationkey"])
    sl = oops.hash_join(ns, t["lineitem"], "s_suppkey", "l_suppkey", ["s_nationkey", "l_price"])
    want = oops.group_by(sl, ["s_nationkey"], [ops.aggregate("SUM", "rev", col("l_price")), ops.aggregate("COUNT", "n")])
    assert got.sorted_rows() == want.sorted_rows()
    # the region filter reached the lineitem side through two filters
    assert any("_bf_use_fw" in o["name"] and o["bloomFilterColumn"] == "l_suppkey" for o in p.ops)
