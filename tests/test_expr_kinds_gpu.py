"""The Like, Substr, DateExtract, DateAdd and If expressions
(fpdb-expression-gandiva/include/fpdb/expression/gandiva/ExpressionType.h:12,29-34)
on the GPU path against the oracle's restatement (oracle.expr): in filter
predicates, in aggregate inputs and as projected columns (Substr as a utf8
column)."""

import numpy as np
import pytest

from flexpushdowndb_gb300 import ops, plan
from flexpushdowndb_gb300.expression import (and_, col, date_add, date_extract, eq, gt, gte, if_, in_, like, lt,
                                             not_, num_lit, or_, str_lit, substr, times)
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops

pytestmark = pytest.mark.gpu

TYPES = ["PROMO BRUSHED TIN", "STANDARD POLISHED BRASS", "PROMO ANODIZED STEEL", "ECONOMY BURNISHED COPPER",
         "MEDIUM PLATED NICKEL", "", "P", "PROMO", "a_b%c", "SMALL BRUSHED BRASS"]


def table(n, seed):
    rng = np.random.default_rng(seed)
    # dates from 1899 to 2030 (negative days included), leap days among them
    days = rng.integers(-25567, 21915, n)
    days[: min(n, 4)] = [11016, -1, 0, 19782][: min(n, 4)]  # 2000-02-29, 1969-12-31, 1970-01-01, 2024-02-29
    return Table([Column("t", "utf8", [TYPES[i] for i in rng.integers(0, len(TYPES), n)]),
                  Column("d", "date32", days),
                  Column("q", "int32", rng.integers(1, 50, n)),
                  Column("p", "int64", rng.integers(100, 100_000, n)),
                  Column("f", "float64", np.round(rng.normal(0, 100, n), 2))])


PREDICATES = [
    like(col("t"), "PROMO%"),
    like(col("t"), "%BRASS"),
    like(col("t"), "%BRUSH%"),
    like(col("t"), "_R%"),
    like(col("t"), "%"),
    like(col("t"), ""),
    like(col("t"), "P"),
    like(col("t"), "a_b%c"),
    not_(like(col("t"), "%E%E%")),
    eq(substr(col("t"), 1, 5), str_lit("PROMO")),
    eq(substr(col("t"), 10, 3), str_lit("BRU")),
    eq(substr(col("t"), -2, 4), str_lit("P")),  # positions -2..1: the first byte
    eq(substr(col("t"), 30, 5), str_lit("")),
    in_(substr(col("t"), 1, 2), ["PR", "EC", "SM"], "utf8"),
    eq(date_extract(col("d"), "Year"), num_lit(1995, "int64")),
    and_(gte(date_extract(col("d"), "Month"), num_lit(6, "int64")), lt(date_extract(col("d"), "Day"), num_lit(10, "int64"))),
    eq(date_extract(col("d"), "Day"), num_lit(29, "int64")),
    lt(col("d"), date_add(num_lit(9131, "date32"), num_lit(3, "int32"), "Month")),  # before 1995-04-01
    gt(date_add(col("d"), num_lit(1, "int32"), "Year"), num_lit(10957, "date32")),
    eq(date_add(col("d"), num_lit(-1, "int64"), "Month"), col("d")),  # never true
    gt(if_(like(col("t"), "PROMO%"), col("p"), num_lit(0, "int64")), num_lit(50_000, "int64")),
    or_(lt(if_(gt(col("q"), num_lit(25)), col("f"), times(col("f"), num_lit(-1.0, "float64"))), num_lit(0.0, "float64")),
        like(col("t"), "%NICKEL")),
]


@pytest.mark.parametrize("n", [0, 1, 5000, 100_003])
@pytest.mark.parametrize("pi", range(len(PREDICATES)))
def test_filter_expressions_match_oracle(gpu, n, pi):
    t = table(n, seed=n + pi)
    pred = PREDICATES[pi]
    got = ops.Filter(pred, t).evaluate(t)
    want = oops.filter_table(t, pred)
    assert got.rows() == want.rows()


def test_group_with_if_aggregate(gpu):
    """SUM(CASE WHEN t LIKE 'PROMO%' THEN p * q ELSE 0 END) per year, the shape
    of TPC-H Q14's promo revenue."""
    t = table(200_000, seed=4)
    aggs = [ops.aggregate("SUM", "promo", if_(like(col("t"), "PROMO%"), times(col("p"), col("q")), num_lit(0, "int64"))),
            ops.aggregate("SUM", "all", times(col("p"), col("q"))), ops.aggregate("COUNT", "n")]
    p = plan.Plan()
    p.scan("scan", "t")
    p.project("proj", "scan", exprs=[("y", date_extract(col("d"), "Year"))], pairs=[("t", "t"), ("p", "p"), ("q", "q")])
    p.group("g", "proj", ["y"], aggs)
    p.collate("collate", "g")
    got = plan.execute(p, {"t": t}).table
    projected = oops.project(t, [("y", date_extract(col("d"), "Year"))], [("t", "t"), ("p", "p"), ("q", "q")])
    want = oops.group_by(projected, ["y"], aggs)
    assert got.sorted_rows() == want.sorted_rows()


@pytest.mark.parametrize("chunk", [0, 30_000])
def test_project_new_expressions(gpu, chunk):
    t = table(70_000, seed=9)
    exprs = [("yr", date_extract(col("d"), "Year")), ("mo", date_extract(col("d"), "Month")),
             ("next_month", date_add(col("d"), num_lit(1, "int32"), "Month")),
             ("prev_year", date_add(col("d"), num_lit(-1, "int32"), "Year")),
             ("tomorrow", date_add(col("d"), num_lit(1, "int32"), "Day")),
             ("promo", if_(like(col("t"), "PROMO%"), num_lit(1, "int32"), num_lit(0, "int32"))),
             ("head", substr(col("t"), 1, 5)), ("mid", substr(col("t"), 7, 4)), ("copy", col("t"))]
    p = plan.Plan()
    p.scan("scan", "t", chunk_rows=chunk)
    p.project("proj", "scan", exprs=exprs, pairs=[("q", "q")])
    p.collate("collate", "proj")
    got = plan.execute(p, {"t": t}).table
    want = oops.project(t, exprs, [("q", "q")])
    assert got.names == want.names
    assert [c.type for c in got.columns] == [c.type for c in want.columns]
    assert got.rows() == want.rows()
