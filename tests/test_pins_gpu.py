"""The reference's own known answers, run on the CUDA path through the C ABI.

tests/test_oracle_pins.py checks the oracle against the same restated
cases; here every case goes through the library's kernels instead: the CSV
parser (gfpdb_csv_read), the selection kernel (gfpdb_filter_evaluate), the
group-by kernels (gfpdb_group_*) and the hash join (gfpdb_hashjoin_*).

The second half pins the workloads at their full sizes against fixtures
written by Arrow's own engine (tests/golden/make_golden.py --full): the
two-table query at 1,000,000 fact rows, the star query at 6,000,000, the CSV
scan of 6,000,000 lineitem rows and the batched form's 32 query variants over
its 64 fact partitions (59,952,713 rows).
"""

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from flexpushdowndb_gb300 import ops, workloads
from flexpushdowndb_gb300.expression import cast, col, eq, lt, num_lit, times
from flexpushdowndb_gb300.ops import aggregate
from flexpushdowndb_gb300.tupleset import Column, DeviceTable, Table

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"

# fpdb-expression-gandiva/test/TestUtil.h:25-45: columns a, b, c = "1".."3", "4".."6", "7".."9"
ABC_CSV = b"1,4,7\n2,5,8\n3,6,9\n"
ABC_FIELDS = [("a", "int64"), ("b", "int64"), ("c", "int64")]
# fpdb-executor/ATTIC/test/data/group/a.csv and .../join/b.csv
GROUP_A = b"aa,ab,ac\n10,13,16\n10,14,17\n12,15,18\n"
JOIN_B = b"ba,bb,bc\n10,23,26\n11,24,27\n10,25,28\n"


def abc_table():
    """The three-row test table, parsed by the GPU CSV reader."""
    return ops.csv_read(ABC_CSV, ABC_FIELDS)


def per_row(table, key, expr, function="SUM"):
    """expr evaluated per row inside the group-by kernel (the key column is
    unique, so each group holds one row): {key: value}."""
    g = ops.Group([key], [aggregate(function, "v", expr)])
    g.group(DeviceTable.from_host(table))
    out = g.finalise()
    return dict(zip(out[key].tolist(), out["v"].tolist())), out.column("v").type


def test_pin_csv_abc_table(gpu):
    t = abc_table()
    assert t.names == ["a", "b", "c"]
    assert t.rows() == [(1, 4, 7), (2, 5, 8), (3, 6, 9)]


def test_pin_multiply_known_products(gpu):
    # fpdb-expression-gandiva/test/MultiplyTest.cpp:35-52: a*b as float64 = 4, 10, 18
    vals, ty = per_row(abc_table(), "a", times(cast(col("a"), "float64"), cast(col("b"), "float64")))
    assert ty == "float64"
    assert vals == {1: 4.0, 2: 10.0, 3: 18.0}


def test_pin_less_than_truth_table(gpu):
    # fpdb-expression-gandiva/test/BinaryExpressionTest.cpp:35-57: cast(x, int32) < k is
    # true on the first row only, for (a, 2), (b, 5), (c, 8)
    t = abc_table()
    dev = DeviceTable.from_host(t)
    for name, k in (("a", 2), ("b", 5), ("c", 8)):
        f = ops.Filter(lt(cast(col(name), "int32"), num_lit(k, "int32")), t)
        sel = f.evaluate(dev)
        assert sel.rows() == [(1, 4, 7)], name


@pytest.mark.parametrize("ty", ["int32", "int64", "float64"])
def test_pin_cast_values(gpu, ty):
    # fpdb-expression-gandiva/test/CastTest.cpp:81-137: a[0]=1, b[1]=5, c[2]=9 after the cast
    t = abc_table()
    for name, key, want in (("a", 1, 1), ("b", 2, 5), ("c", 3, 9)):
        vals, _ = per_row(t, "a", cast(col(name), ty), function="MAX")
        assert vals[key] == want
    # the cast inside a predicate selects the same row
    dev = DeviceTable.from_host(t)
    lit = num_lit(5.0, "float64") if ty == "float64" else num_lit(5, ty)
    sel = ops.Filter(eq(cast(col("b"), ty), lit), t).evaluate(dev)
    assert sel.rows() == [(2, 5, 8)]


def test_pin_csv_test_file(gpu):
    # fpdb-tuple/data/csv/test.csv as fpdb-tuple/test/CSVTest.cpp:35-79,192 describes it:
    # header A,B,C then rows 1,2,3 / 4,5,6 / 7,8,9; 24 bytes; read whole, then two columns.
    text = b"A,B,C\n1,2,3\n4,5,6\n7,8,9\n"
    assert len(text) == 24
    fields = [("a", "utf8"), ("b", "utf8"), ("c", "utf8")]
    t = ops.csv_read(text, fields, has_header=True)
    assert t.rows() == [("1", "2", "3"), ("4", "5", "6"), ("7", "8", "9")]
    t2 = ops.csv_read(text, fields, columns=["a", "b"], has_header=True)
    assert t2.names == ["a", "b"] and t2.rows() == [("1", "2"), ("4", "5"), ("7", "8")]


def test_pin_csv_3x10000(gpu):
    # fpdb-tuple/data/csv/test3x10000.csv per CSVTest.cpp:203: header, then
    # 10000 rows cycling 1,2,3 / 4,5,6 / 7,8,9; 60006 bytes.
    rows = [b"1,2,3\n", b"4,5,6\n", b"7,8,9\n"]
    text = b"A,B,C\n" + b"".join(rows[r % 3] for r in range(10000))
    assert len(text) == 60006
    t = ops.csv_read(text, [("a", "int32"), ("b", "int32"), ("c", "int32")], has_header=True)
    assert t.num_rows == 10000
    a = t["a"]
    assert a[0] == 1 and a[1] == 4 and a[2] == 7 and a[9999] == 1
    assert int(t["c"].sum()) == 3 * 3334 + 6 * 3333 + 9 * 3333  # c cycles 3, 6, 9


def test_pin_attic_group_sum(gpu):
    # fpdb-executor/ATTIC/test/GroupTest.cpp:137-150: group by AA, sum(AB) -> 10: 27, 12: 15
    t = ops.csv_read(GROUP_A, [("aa", "int64"), ("ab", "int64"), ("ac", "int64")], has_header=True)
    g = ops.Group(["aa"], [aggregate("SUM", "sum", col("ab"))])
    g.group(DeviceTable.from_host(t))
    assert g.finalise().sorted_rows() == [(10, 27), (12, 15)]


def test_pin_attic_join(gpu):
    # fpdb-executor/ATTIC/test/JoinTest.cpp:82-123: a join b on aa = ba -> 4 rows,
    # probe side (a) columns first, then the build side's (b)
    a = ops.csv_read(GROUP_A, [("aa", "int64"), ("ab", "int64"), ("ac", "int64")], has_header=True)
    b = ops.csv_read(JOIN_B, [("ba", "int64"), ("bb", "int64"), ("bc", "int64")], has_header=True)
    j = ops.HashJoin("ba", "aa")
    j.put_build(DeviceTable.from_host(b))
    j.finalize_build()
    out = j.probe(DeviceTable.from_host(a))
    assert out.names == ["aa", "ab", "ac", "ba", "bb", "bc"]
    assert out.sorted_rows() == sorted([
        (10, 13, 16, 10, 23, 26), (10, 13, 16, 10, 25, 28), (10, 14, 17, 10, 23, 26), (10, 14, 17, 10, 25, 28)])


def test_pin_int32_multiply_wraps(gpu):
    # Gandiva's multiply(int32, int32) returns int32 (BinaryExpression.cpp:57-102),
    # so the product wraps before the int64 sum
    t = Table([Column("x", "int32", [70000, -3]), Column("y", "int32", [70000, 5])])
    vals, _ = per_row(t, "x", times(col("x"), col("y")))
    assert vals == {70000: int(np.int32(np.int64(70000 * 70000) - 2**32)), -3: -15}


def test_pin_bloom_no_false_negatives_and_fpr(gpu):
    from oracle import ops as oops

    rng = np.random.default_rng(7)
    keys = rng.choice(10**7, size=20000, replace=False)
    bf = ops.BloomFilter([Table([Column("k", "int64", keys)])], "k", bits_per_key=10, num_hashes=3)
    assert np.array_equal(bf.words(), oops.bloom_words(keys, 10, 3))
    others = np.setdiff1d(rng.choice(10**7, size=200000, replace=False), keys)
    probe = Table([Column("k", "int64", np.concatenate([keys, others]))])
    kept = bf.use(DeviceTable.from_host(probe), "k")["k"]
    assert np.isin(keys, kept).all()  # no false negatives
    assert (len(kept) - len(keys)) / len(others) < 0.035


# ------------------------------------------------------------- full sizes


def fixture(name):
    p = GOLDEN / f"{name}.json"
    return json.loads(p.read_text())


def rows(x):
    return sorted(tuple(r) for r in x)


def digest(rs):
    h = hashlib.sha256()
    for r in rs:
        h.update((",".join(str(v) for v in r) + "\n").encode())
    return h.hexdigest()


def test_full_two_table_1m(gpu):
    """The plain two-table query at its full 1,000,000 fact rows."""
    from flexpushdowndb_gb300 import plan

    f = fixture("two_table_1m")
    t = workloads.two_table_tables(fact_rows=f["fact_rows"], seed=f["seed"])
    assert f["fact_rows"] == 1_000_000
    for graph in (False, True):
        text = json.loads(workloads.two_table_plan().to_json())
        text["cudaGraph"] = graph
        assert plan.execute(json.dumps(text), t).table.sorted_rows() == rows(f["rows"])


def test_full_star_6m(gpu):
    """The star query with bloom predicate transfer at its full 6,000,000 fact rows."""
    from flexpushdowndb_gb300 import plan

    f = fixture("star_6m")
    assert f["fact_rows"] == 6_000_000
    t = workloads.star_tables(fact_rows=f["fact_rows"], seed=f["seed"])
    got = plan.execute(workloads.star_plan(consts=tuple(f["consts"])), t).table.sorted_rows()
    assert got == rows(f["rows"])


def test_full_csv_scan_6m(gpu):
    """The CSV ingest of 6,000,000 lineitem rows (every column's sum and
    every string column's digest) and the scan plan over the same text."""
    from flexpushdowndb_gb300 import plan
    from flexpushdowndb_gb300.tupleset import text_table

    f = fixture("csv_scan_6m")
    text = workloads.lineitem_csv(f["rows"], f["seed"], processes=8)
    assert len(text) == f["text_bytes"]
    t = ops.csv_read(text, workloads.LINEITEM_FIELDS, delimiter="|")
    assert t.num_rows == f["rows"]
    for n, v in f["column_sums"].items():
        assert int(np.asarray(t[n], dtype=np.int64).sum()) == v, n
    for n, d in f["string_digests"].items():
        assert digest([(s,) for s in t.column(n).to_list()]) == d, n
    del t
    got = plan.execute(workloads.csv_scan_plan(), {"lineitem": text_table(text)}).table
    assert got.rows() == [(f["sum_d2_i2"], f["selected"])]


def test_full_star_batch_64x32(gpu):
    """The batched form at full size: 32 query variants over 64 fact
    partitions in one gfpdb_star_batch call, graph captured and replayed;
    every variant's groups against Arrow's."""
    from flexpushdowndb_gb300 import batch, plan

    f = fixture("star_batch_64x32")
    tabs = workloads.batch_tables(f["parts"])
    parts = [f"p{i}" for i in range(f["parts"])]
    assert sum(tabs[p].num_rows for p in parts) == f["fact_rows"]
    dev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
    qs = [[tuple(r) for r in v["ranges"]] for v in f["variants"]]
    spec = workloads.star_batch_spec(parts, qs)
    for _ in range(3):  # first run, capture, replay
        got = batch.split_by_query(batch.star_batch(spec, dev).table)
    for q, v in enumerate(f["variants"]):
        r = got.get(q, [])
        assert len(r) == v["groups"], q
        assert sum(x[2] for x in r) == v["sum_revenue"], q
        assert sum(x[4] for x in r) == v["sum_cnt"], q
        assert digest(r) == v["digest"], q
    batch.clear_graph_cache()
