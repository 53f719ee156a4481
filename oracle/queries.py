"""The two-table and star queries composed from the oracle operators
(TEST INFRASTRUCTURE ONLY).

The star query applies the same forward + backward bloom predicate transfer
as the plan (SmallToLargePredTransOrder.cpp:38-214) with the oracle's bloom;
blooms only remove rows that cannot join, so the result equals the plain
filtered 4-way join, which star_query_direct computes without blooms as a
cross-check.
"""

from __future__ import annotations

from flexpushdowndb_gb300.expression import col, eq, lt, num_lit, times
from flexpushdowndb_gb300.tupleset import Table

from . import ops

REVENUE = times(col("price_cents"), col("qty"))
DISC_REVENUE = times(col("price_cents"), col("discount"))


def two_table_query(tables: dict[str, Table], category_lt: int = 5) -> Table:
    dim = ops.filter_table(tables["dim"], lt(col("category"), num_lit(category_lt, "int32")), ["pk", "region"])
    fact = tables["fact"]
    j = ops.hash_join(dim, fact, "pk", "fk", ["region", "qty", "price_cents"])
    return ops.group_by(j, ["region"], [{"function": "SUM", "name": "revenue", "expr": REVENUE},
                                        {"function": "COUNT", "name": "cnt"}])


def _star_dims(tables, consts):
    out = {}
    for i in range(1, 5):
        keep = [f"d{i}_pk", f"d{i}_g"] if i in (2, 4) else [f"d{i}_pk"]
        out[i] = ops.filter_table(tables[f"d{i}"], eq(col(f"d{i}_f"), num_lit(int(consts[i - 1]), "int32")), keep)
    return out


def _star_join_group(fact: Table, dims: dict[int, Table]) -> Table:
    cur = fact
    fact_cols = ["fk1", "fk2", "fk3", "fk4", "qty", "price_cents", "discount"]
    carried: list[str] = []
    for i in range(1, 5):
        fact_cols = [c for c in fact_cols if c != f"fk{i}"]
        if i in (2, 4):
            carried.append(f"d{i}_g")
        cur = ops.hash_join(dims[i], cur, f"d{i}_pk", f"fk{i}", fact_cols + carried)
    return ops.group_by(cur, ["d2_g", "d4_g"], [
        {"function": "SUM", "name": "revenue", "expr": REVENUE},
        {"function": "SUM", "name": "discount_revenue", "expr": DISC_REVENUE},
        {"function": "COUNT", "name": "cnt"},
    ])


def star_query(tables: dict[str, Table], consts=(1, 3, 2, 5), bits_per_key: int = 10, num_hashes: int = 3,
               stats: dict | None = None) -> Table:
    dims = _star_dims(tables, consts)
    fact = tables["fact"]
    for i in (2, 3, 4, 1):  # forward pass
        w = ops.bloom_words(dims[i][f"d{i}_pk"], bits_per_key, num_hashes)
        fact = ops.bloom_use(fact, w, f"fk{i}", num_hashes)
    for i in range(1, 5):  # backward pass
        w = ops.bloom_words(fact[f"fk{i}"], bits_per_key, num_hashes)
        dims[i] = ops.bloom_use(dims[i], w, f"d{i}_pk", num_hashes)
    if stats is not None:
        stats["fact_after_forward"] = fact.num_rows
        stats["dims_after_backward"] = [dims[i].num_rows for i in range(1, 5)]
    return _star_join_group(fact, dims)


def star_query_direct(tables: dict[str, Table], consts=(1, 3, 2, 5)) -> Table:
    return _star_join_group(tables["fact"], _star_dims(tables, consts))


def concat_tables(parts: list[Table]) -> Table:
    import numpy as np

    from flexpushdowndb_gb300.tupleset import Column

    return Table([Column(c.name, c.type, np.concatenate([p.column(c.name).values for p in parts]))
                  for c in parts[0].columns])


def star_query_ranges(tables: dict[str, Table], fact_tables, ranges) -> Table:
    """The star query with lo <= d{i}_f <= hi dimension filters over a fact
    table given as partitions (no bloom pass: blooms never change results)."""
    from flexpushdowndb_gb300.expression import and_, gte, lte

    dims = {}
    for i in range(1, 5):
        keep = [f"d{i}_pk", f"d{i}_g"] if i in (2, 4) else [f"d{i}_pk"]
        lo, hi = ranges[i - 1]
        pred = and_(gte(col(f"d{i}_f"), num_lit(int(lo), "int32")), lte(col(f"d{i}_f"), num_lit(int(hi), "int32")))
        dims[i] = ops.filter_table(tables[f"d{i}"], pred, keep)
    fact = concat_tables([tables[t] for t in fact_tables])
    return _star_join_group(fact, dims)
