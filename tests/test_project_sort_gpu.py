"""ProjectPOp and LimitSortPOp on the GPU path, against the oracle's
restatements (oracle.ops.project / limit_sort), inside physical plans."""

import json

import numpy as np
import pytest

from flexpushdowndb_gb300 import GfpdbError, plan, workloads
from flexpushdowndb_gb300.expression import cast, col, divide, gt, num_lit, times
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops
from oracle import queries

pytestmark = pytest.mark.gpu


def star_top(k, keys, graph=False):
    p = workloads.star_plan()
    d = json.loads(p.to_json())
    # the group-by's consumer becomes a LimitSortPOp that feeds the collate
    for o in d["ops"]:
        if o["type"] == "GroupPOp":
            o["consumers"] = ["top"]
    d["ops"] = [o for o in d["ops"] if o["type"] != "CollatePOp"]
    d["ops"].append({"type": "LimitSortPOp", "name": "top", "k": k,
                     "sortKeys": [{"name": n, "order": o} for n, o in keys], "consumers": ["collate"]})
    d["ops"].append({"type": "CollatePOp", "name": "collate"})
    d["cudaGraph"] = graph
    return json.dumps(d)


@pytest.mark.parametrize("graph", [False, True])
def test_star_query_top_groups(gpu, graph):
    """ORDER BY revenue DESC, cnt, d2_g, d4_g LIMIT 10 over the star query's groups."""
    tabs = workloads.star_tables(fact_rows=300_000, seed=2017)
    keys = [("revenue", "DESC"), ("cnt", "ASC"), ("d2_g", "ASC"), ("d4_g", "ASC")]
    want = oops.limit_sort(queries.star_query(tabs), 10, keys).rows()
    for _ in range(3 if graph else 1):
        got = plan.execute(star_top(10, keys, graph), tabs).table
        assert got.names == ["d2_g", "d4_g", "revenue", "discount_revenue", "cnt"]
        assert got.rows() == want


def sort_table(n, seed):
    rng = np.random.default_rng(seed)
    words = [f"w{i:03d}" for i in range(40)]
    return Table([Column("a", "int64", rng.integers(-50, 50, n)),
                  Column("f", "float64", np.round(rng.normal(0, 10, n), 1)),
                  Column("s", "utf8", [words[i] for i in rng.integers(0, 40, n)]),
                  Column("row", "int32", np.arange(n))])


@pytest.mark.parametrize("n,k,keys", [
    (100_003, 1000, [("a", "ASC")]),                     # many rounds, heavy ties (input order kept)
    (70_000, 64, [("s", "DESC"), ("a", "ASC")]),         # utf8 first key
    (5_000, 1024, [("f", "DESC"), ("s", "ASC")]),        # float64 key, the largest k
    (37, 100, [("a", "DESC")]),                          # k above the row count
    (0, 10, [("a", "ASC")]),                             # no rows
])
def test_limit_sort_matches_oracle(gpu, n, k, keys):
    t = sort_table(n, seed=n + k)
    p = plan.Plan()
    p.scan("scan", "t")
    p.limit_sort("top", "scan", k, keys)
    p.collate("collate", "top")
    got = plan.execute(p, {"t": t}).table
    assert got.rows() == oops.limit_sort(t, k, keys).rows()


def test_limit_sort_rejects_large_k_and_bad_order(gpu):
    for k, order in ((1025, "ASC"), (10, "UP")):
        p = plan.Plan()
        p.scan("scan", "t")
        p.limit_sort("top", "scan", k, [("a", order)])
        p.collate("collate", "top")
        with pytest.raises(GfpdbError):
            plan.execute(p, {"t": sort_table(10, 1)})


@pytest.mark.parametrize("graph", [False, True])
def test_project_after_group_and_after_filter(gpu, graph):
    """Pass-through columns renamed, then expressions: integer division,
    float arithmetic, int32 * int32 (wrapping); once over a group-by's output
    and once over a filter's (deferred-size) output."""
    tabs = workloads.two_table_tables(fact_rows=200_000, seed=1003)
    p = json.loads(workloads.two_table_plan().to_json())
    for o in p["ops"]:
        if o["type"] == "GroupPOp":
            o["consumers"] = ["proj"]
    p["ops"] = [o for o in p["ops"] if o["type"] != "CollatePOp"]
    exprs = [("avg_rev", divide(col("revenue"), col("cnt"))),
             ("half", times(cast(col("revenue"), "float64"), num_lit(0.5, "float64")))]
    pairs = [("region", "r"), ("cnt", "n")]
    p["ops"].append({"type": "ProjectPOp", "name": "proj", "exprs": [{"name": n, "expr": e} for n, e in exprs],
                     "projectColumnNamePairs": [list(x) for x in pairs], "consumers": ["collate"]})
    p["ops"].append({"type": "CollatePOp", "name": "collate"})
    p["cudaGraph"] = graph
    want = oops.project(queries.two_table_query(tabs), exprs, pairs).sorted_rows()
    for _ in range(3 if graph else 1):
        got = plan.execute(json.dumps(p), tabs).table
        assert got.names == ["r", "n", "avg_rev", "half"]
        assert got.sorted_rows() == want
    # over a filter's output
    fact = tabs["fact"]
    q = plan.Plan()
    q.scan("scan", "fact")
    q.filter("f", "scan", gt(col("qty"), num_lit(40)), ["fk", "qty", "price_cents"])
    q.project("proj", "f", [("q2", times(col("qty"), col("qty"))), ("pq", times(col("price_cents"), col("qty")))],
              [("fk", "key")])
    q.collate("collate", "proj")
    got = plan.execute(q, {"fact": fact}).table
    sel = oops.filter_table(fact, gt(col("qty"), num_lit(40)), ["fk", "qty", "price_cents"])
    want = oops.project(sel, [("q2", times(col("qty"), col("qty"))), ("pq", times(col("price_cents"), col("qty")))],
                        [("fk", "key")])
    assert got.rows() == want.rows()
