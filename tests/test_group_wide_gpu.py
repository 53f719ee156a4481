"""Group-bys whose keys do not pack into 64 bits (three to eight columns, or
two int64 columns): keys grouped through the device record dictionary, against
the oracle's group_by, across batches and inside plans."""

import numpy as np
import pytest

from flexpushdowndb_gb300 import GfpdbError, ops, plan
from flexpushdowndb_gb300.expression import col, times
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def wide_table(n, seed, card=6):
    rng = np.random.default_rng(seed)
    words = ["", "a", "bb", "ccc", "dddd", "a b"]
    return Table([Column("i", "int32", rng.integers(-card, card, n)),
                  Column("l", "int64", rng.integers(0, card, n) * (2**40) - 7),
                  Column("d", "date32", rng.integers(9000, 9000 + card, n)),
                  Column("s", "utf8", [words[k] for k in rng.integers(0, len(words), n)]),
                  Column("m", "int64", rng.integers(-(2**50), 2**50, n)),
                  Column("v", "int32", rng.integers(-100, 100, n))])


AGGS = [ops.aggregate("SUM", "sm", col("m")), ops.aggregate("COUNT", "cnt"), ops.aggregate("MIN", "lo", col("v")),
        ops.aggregate("MAX", "hi", col("m")), ops.aggregate("AVG", "av", col("v")),
        ops.aggregate("SUM", "iv", times(col("i"), col("v")))]


@pytest.mark.parametrize("keys", [["i", "l", "d"], ["l", "m"], ["s", "l", "i"], ["i", "d", "s", "l", "v"],
                                  ["i", "l", "d", "s", "v", "m"]])
@pytest.mark.parametrize("sizes", [(0,), (1,), (5000,), (70_000, 1, 30_000)])
def test_wide_keys_match_oracle(gpu, keys, sizes):
    batches = [wide_table(n, seed=17 * (i + 1) + n) for i, n in enumerate(sizes)]
    g = ops.Group(keys, AGGS)
    for b in batches:
        g.group(b)
    got = g.finalise()
    whole = Table.concat(batches) if len(batches) > 1 else batches[0]
    want = oops.group_by(whole, keys, AGGS)
    assert got.names == want.names
    assert [c.type for c in got.columns] == [c.type for c in want.columns]
    assert got.sorted_rows() == want.sorted_rows()


def test_wide_keys_many_groups(gpu):
    """300K rows over ~200K distinct three-column keys: the record dictionary
    and the table grow across batches."""
    n = 300_000
    rng = np.random.default_rng(5)
    t = Table([Column("a", "int32", rng.integers(0, 100, n)), Column("b", "int32", rng.integers(0, 100, n)),
               Column("c", "int32", rng.integers(0, 50, n)), Column("v", "int64", rng.integers(0, 1000, n))])
    aggs = [ops.aggregate("SUM", "s", col("v")), ops.aggregate("COUNT", "n")]
    g = ops.Group(["a", "b", "c"], aggs)
    for lo in range(0, n, 100_000):
        g.group(t.slice(lo, lo + 100_000))
    got = g.finalise()
    want = oops.group_by(t, ["a", "b", "c"], aggs)
    assert got.num_rows == want.num_rows
    assert got.sorted_rows() == want.sorted_rows()


def test_wide_keys_in_a_plan(gpu):
    t = wide_table(40_000, seed=3)
    p = plan.Plan()
    p.scan("scan", "t", chunk_rows=15_000)
    p.group("g", "scan", ["s", "i", "d"], AGGS)
    p.collate("collate", "g")
    got = plan.execute(p, {"t": t}).table
    assert got.sorted_rows() == oops.group_by(t, ["s", "i", "d"], AGGS).sorted_rows()


def test_eight_key_columns(gpu):
    rng = np.random.default_rng(8)
    n = 20_000
    cols = [Column(f"k{i}", "int64" if i % 3 == 0 else "int32", rng.integers(0, 3, n)) for i in range(8)]
    t = Table(cols + [Column("v", "int64", rng.integers(0, 10, n))])
    keys = [c.name for c in cols]
    aggs = [ops.aggregate("SUM", "s", col("v")), ops.aggregate("COUNT", "n")]
    g = ops.Group(keys, aggs)
    g.group(t)
    assert g.finalise().sorted_rows() == oops.group_by(t, keys, aggs).sorted_rows()


def test_more_than_eight_key_columns_is_rejected(gpu):
    cols = [Column(f"k{i}", "int32", [1, 2]) for i in range(9)]
    g = ops.Group([c.name for c in cols], [ops.aggregate("COUNT", "n")])
    with pytest.raises(GfpdbError):
        g.group(Table(cols))
