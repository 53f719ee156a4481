"""The device shuffle (gfpdb_shuffle, ShufflePOp) and the two-phase group-by
built on it, against the oracle's restatements (oracle.ops.shuffle /
group_by): the same rows in the same slots and order, bit for bit, at sizes
the oracle finishes quickly; at larger sizes, properties that do not need the
oracle's row-by-row output (every row once, each slot's rows hash there,
input order kept within a slot)."""

import numpy as np
import pytest

from flexpushdowndb_gb300 import GfpdbError, ops, plan, workloads
from flexpushdowndb_gb300.expression import col, num_lit, times
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def mixed_table(n, seed, n_keys=50):
    rng = np.random.default_rng(seed)
    words = [f"k{i}" * (1 + i % 3) for i in range(n_keys)]
    return Table([Column("a", "int32", rng.integers(0, n_keys, n)),
                  Column("b", "int64", rng.integers(-(2**40), 2**40, n)),
                  Column("d", "date32", rng.integers(8000, 9000, n)),
                  Column("s", "utf8", [words[i] for i in rng.integers(0, n_keys, n)]),
                  Column("f", "float64", rng.normal(0, 1, n)),
                  Column("row", "int32", np.arange(n))])


@pytest.mark.parametrize("n", [0, 1, 31, 33, 1000, 100_003])
@pytest.mark.parametrize("keys,slots", [
    (["a"], 7), (["b"], 64), (["s"], 5), (["a", "s"], 16), (["d", "b"], 1), (["a"], 1000), (["b"], 1024),
])
def test_shuffle_matches_oracle(gpu, n, keys, slots):
    t = mixed_table(n, seed=n + slots)
    got, offs = ops.shuffle(t, keys, slots)
    want, woffs = oops.shuffle(t, keys, slots)
    assert offs == woffs
    assert got.names == t.names
    assert got.rows() == want.rows()


def test_shuffle_split_is_slices(gpu):
    t = mixed_table(5000, seed=3)
    parts = ops.shuffle_split(t, ["s", "a"], 9)
    want, offs = oops.shuffle(t, ["s", "a"], 9)
    assert [p.num_rows for p in parts] == [offs[i + 1] - offs[i] for i in range(9)]
    assert sum((p.rows() for p in parts), []) == want.rows()


def test_int32_and_int64_keys_share_slots(gpu):
    """Integer keys hash by value, so the two sides of a join on an int32 and
    an int64 column partition alike."""
    v = np.arange(-500, 500)
    a, oa = ops.shuffle(Table([Column("k", "int32", v)]), ["k"], 13)
    b, ob = ops.shuffle(Table([Column("k", "int64", v)]), ["k"], 13)
    assert oa == ob and a["k"].tolist() == b["k"].tolist()


def test_shuffle_at_scale(gpu):
    """20M rows over 256 slots: the slots hold every row once, each row sits
    in the slot its key hashes to, and input order is kept within a slot."""
    n, slots = 20_000_000, 256
    rng = np.random.default_rng(11)
    keys = workloads.zipf_keys(n, 10_000_000, seed=11)
    t = Table([Column("k", "int64", keys), Column("v", "int32", rng.integers(0, 1000, n)),
               Column("row", "int32", np.arange(n))])
    got, offs = ops.shuffle(t, ["k"], slots)
    assert offs[0] == 0 and offs[-1] == n and all(offs[i] <= offs[i + 1] for i in range(slots))
    row = got["row"]
    assert np.array_equal(np.sort(row), np.arange(n))
    slot_of_row = oops.shuffle_slots(Table([Column("k", "int64", got["k"])]), ["k"], slots)
    assert np.array_equal(slot_of_row, np.repeat(np.arange(slots), np.diff(offs)))
    assert np.array_equal(got["k"], keys[row]) and np.array_equal(got["v"], t["v"][row])
    inner = np.diff(row.astype(np.int64))
    boundary = np.zeros(n - 1, dtype=bool)
    ends = np.array(offs[1:-1]) - 1
    boundary[ends[(ends >= 0) & (ends < n - 1)]] = True
    assert (inner[~boundary] > 0).all()


def test_shuffle_argument_errors(gpu):
    t = mixed_table(10, seed=1)
    for keys, slots in ((["a"], 0), (["a"], 1025), (["f"], 4), (["missing"], 4)):
        with pytest.raises(GfpdbError):
            ops.shuffle(t, keys, slots)


# ----------------------------------------------------------- plan operators


def two_phase_plan(n_parts, degree, aggregates, group_columns):
    p = plan.Plan()
    scans = [p.scan(f"scan{i}", f"t{i}") for i in range(n_parts)]
    reduces = p.group_two_phase("g", scans, group_columns, aggregates, degree)
    p._add({"type": "CollatePOp", "name": "collate"})
    for r in reduces:
        p.connect(r, "collate")
    return p


AGGS = [ops.aggregate("SUM", "sum_b", col("b")), ops.aggregate("COUNT", "cnt"),
        ops.aggregate("MIN", "min_b", col("b")), ops.aggregate("MAX", "max_d", col("d")),
        ops.aggregate("AVG", "avg_a", col("a")), ops.aggregate("SUM", "sum_ab", times(col("a"), col("b")))]


@pytest.mark.parametrize("group_columns", [["a"], ["s"], ["a", "d"]])
@pytest.mark.parametrize("n_parts,degree", [(1, 1), (3, 4), (4, 1)])
def test_two_phase_group_matches_one_phase(gpu, group_columns, n_parts, degree):
    tabs = {f"t{i}": mixed_table(20_000 + 7 * i, seed=100 + i) for i in range(n_parts)}
    whole = Table.concat(list(tabs.values())) if n_parts > 1 else tabs["t0"]
    want = oops.group_by(whole, group_columns, AGGS)
    p = two_phase_plan(n_parts, degree, AGGS, group_columns)
    plan.validate(p)
    got = plan.execute(p, tabs).table
    assert got.names == want.names
    assert got.sorted_rows() == want.sorted_rows()


def test_two_phase_high_cardinality_zipf(gpu):
    """The 10M-key Zipf(1.1) int64 group-by in two phases over 4 fact
    partitions and 8 reduce groups equals the one-phase group-by."""
    n = 4_000_000
    keys = workloads.zipf_keys(n, 10_000_000, seed=21)
    vals = np.random.default_rng(21).integers(-1000, 1000, n)
    tabs = {f"t{i}": Table([Column("k", "int64", keys[i::4]), Column("v", "int64", vals[i::4])]) for i in range(4)}
    aggs = [ops.aggregate("SUM", "s", col("v")), ops.aggregate("COUNT", "c")]
    got = plan.execute(two_phase_plan(4, 8, aggs, ["k"]), tabs).table
    one = plan.Plan()
    one.scan("scan", "t")
    one.group("g", "scan", ["k"], aggs)
    one.collate("collate", "g")
    want = plan.execute(one, {"t": Table([Column("k", "int64", keys), Column("v", "int64", vals)])}).table
    assert got.num_rows == want.num_rows
    assert got.sorted_rows() == want.sorted_rows()


def test_shuffle_pop_sends_slot_i_to_consumer_i(gpu):
    t = mixed_table(3000, seed=5)
    p = plan.Plan()
    p.scan("scan", "t", chunk_rows=1000)
    consumers = [f"c{i}" for i in range(3)]
    p.shuffle("sh", "scan", ["s"])
    for i, c in enumerate(consumers):
        p.project(c, "sh", exprs=[("cid", num_lit(i))], pairs=[("row", "row"), ("s", "s")])
    p._add({"type": "CollatePOp", "name": "collate"})
    for c in consumers:
        p.connect(c, "collate")
    got = plan.execute(p, {"t": t}).table
    # every row once; each consumer's rows hash to its slot
    assert sorted(got["row"].tolist()) == list(range(3000))
    assert np.array_equal(oops.shuffle_slots(got, ["s"], 3), got["cid"])
