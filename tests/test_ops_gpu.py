"""Operator parity on the GPU: every kernel path against the oracle, bit-exact.

Filter / select outputs keep input order and are compared row by row; join
and group outputs have no order and are compared as sorted multisets.
"""

import numpy as np
import pytest

from flexpushdowndb_gb300 import GfpdbError, ops, workloads
from flexpushdowndb_gb300.expression import (and_, cast, col, divide, eq, gt, gte, in_, isNull, lt, lte, minus, neq,
                                             not_, num_lit, or_, plus, str_lit, times)
from flexpushdowndb_gb300.tupleset import Column, DeviceTable, Table
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def rand_table(n, seed=1):
    rng = np.random.default_rng(seed)
    return Table([
        Column("i32", "int32", rng.integers(-1000, 1000, n)),
        Column("i64", "int64", rng.integers(-10**12, 10**12, n)),
        Column("d", "date32", rng.integers(8000, 11000, n)),
        Column("f", "float64", rng.normal(0, 100, n)),
        Column("k", "int32", rng.integers(0, 50, n)),
        Column("s", "utf8", [("ab" * int(x))[: int(x) % 7] + str(int(x) % 5) for x in rng.integers(0, 40, n)]),
    ])


PREDICATES = [
    lt(col("i32"), num_lit(0)),
    and_(gte(col("i32"), num_lit(-100)), lt(col("i32"), num_lit(250)), gt(col("d"), num_lit(9000, "date32"))),
    or_(eq(col("k"), num_lit(3)), eq(col("k"), num_lit(7)), lt(col("i64"), num_lit(0, "int64"))),
    not_(and_(lt(col("i32"), num_lit(10)), gt(col("k"), num_lit(20)))),
    in_(col("k"), [1, 2, 3, 40, 41], "int32"),
    not_(in_(col("k"), [1, 2, 3], "int32")),
    gt(col("f"), num_lit(12.5, "float64")),
    lt(times(col("i32"), col("k")), num_lit(-5000, "int64")),
    gt(plus(col("i64"), cast(col("i32"), "int64")), num_lit(0, "int64")),
    lte(minus(col("i32"), col("k")), num_lit(7)),
    eq(divide(col("i32"), num_lit(7)), num_lit(3)),
    eq(col("s"), str_lit("ab3")),
    and_(neq(col("s"), str_lit("0")), lt(col("k"), num_lit(25))),
    in_(col("s"), ["1", "ab2", "abab4"], "utf8"),
    not_(isNull(col("i32"))),
    isNull(col("i32")),
    gt(col("i32"), num_lit(10**6)),  # selects nothing
]


@pytest.mark.parametrize("pi", range(len(PREDICATES)))
@pytest.mark.parametrize("n", [0, 1, 2047, 2048, 2049, 100_003])
def test_filter_parity(gpu, pi, n):
    t = rand_table(n, seed=n + pi)
    pred = PREDICATES[pi]
    f = ops.Filter(pred, t)
    got = f.evaluate(t)
    want = oops.filter_table(t, pred)
    assert got.names == want.names
    assert got.rows() == want.rows()


def test_filter_projection_and_device_input(gpu):
    t = rand_table(50_000, seed=3)
    pred = and_(gt(col("k"), num_lit(10)), lt(col("i32"), num_lit(500)))
    f = ops.Filter(pred, t)
    got = f.evaluate(DeviceTable.from_host(t), project=["s", "i64", "nonexistent"][:2])
    want = oops.filter_table(t, pred, ["s", "i64"])
    assert got.names == ["s", "i64"]
    assert got.rows() == want.rows()


def test_bloom_bits_exact_and_no_false_negatives(gpu):
    rng = np.random.default_rng(11)
    keys = rng.choice(10**7, size=30_000, replace=False).astype(np.int64)
    t = Table([Column("key", "int32", keys)])
    parts = [t.slice(0, 10_000), t.slice(10_000, 30_000)]
    bf = ops.BloomFilter(parts, "key", 10, 3)
    info = bf.info()
    assert info["num_blocks"] == oops.bloom_num_blocks(30_000, 10)
    assert np.array_equal(bf.words(), oops.bloom_words(keys, 10, 3))
    probe = Table([Column("key", "int32", np.concatenate([keys, rng.integers(0, 10**7, 100_000)]))])
    got = bf.use(probe, "key")
    want = oops.bloom_use(probe, oops.bloom_words(keys, 10, 3), "key")
    assert got.rows() == want.rows()
    assert set(keys.tolist()) <= set(got["key"].tolist())


@pytest.mark.parametrize("n_keys", [0, 1, 7, 5000])
def test_bloom_small_and_int64_keys(gpu, n_keys):
    keys = (np.arange(n_keys, dtype=np.int64) * 7919 - 10**10)
    t = Table([Column("k", "int64", keys), Column("v", "int32", np.arange(n_keys))])
    bf = ops.BloomFilter([t], "k", 12, 4)
    assert np.array_equal(bf.words(), oops.bloom_words(keys, 12, 4))
    probe = Table([Column("k", "int64", np.arange(-50, 50, dtype=np.int64) * 7919 - 10**10)])
    got = bf.use(probe, "k")
    assert got.rows() == oops.bloom_use(probe, oops.bloom_words(keys, 12, 4), "k", 4).rows()


def test_select_fused_chain_equals_sequential(gpu):
    tabs = workloads.star_tables(fact_rows=300_000)
    fact = tabs["fact"]
    blooms = []
    seq = fact
    for i, c in ((2, 3), (3, 2), (4, 5), (1, 1)):
        d = oops.filter_table(tabs[f"d{i}"], eq(col(f"d{i}_f"), num_lit(c)))
        blooms.append((ops.BloomFilter([d], f"d{i}_pk"), f"fk{i}"))
        seq = oops.bloom_use(seq, oops.bloom_words(d[f"d{i}_pk"]), f"fk{i}")
    pred = gt(col("qty"), num_lit(10))
    got = ops.select(DeviceTable.from_host(fact), ops.Filter(pred, fact), blooms)
    want = oops.filter_table(seq, pred)
    assert got.rows() == want.rows()


@pytest.mark.parametrize("build_n,probe_n,dup", [(0, 10, 1), (10, 0, 1), (1000, 50_000, 1), (5000, 200_000, 3),
                                                 (200_000, 300_000, 1)])
def test_join_parity(gpu, build_n, probe_n, dup):
    rng = np.random.default_rng(build_n + probe_n)
    bkeys = np.repeat(np.arange(build_n // dup, dtype=np.int64), dup)[:build_n]
    build = Table([Column("pk", "int32", bkeys), Column("bv", "int64", rng.integers(0, 10**9, len(bkeys))),
                   Column("bs", "utf8", [f"s{x % 13}" for x in bkeys])])
    probe = Table([Column("fk", "int32", rng.integers(-5, max(1, build_n // dup) + 5, probe_n)),
                   Column("pv", "int32", rng.integers(0, 100, probe_n))])
    j = ops.HashJoin("pk", "fk")
    j.put_build(build)
    j.finalize_build()
    got = j.probe(DeviceTable.from_host(probe))
    want = oops.hash_join(build, probe, "pk", "fk")
    assert got.names == want.names == ["fk", "pv", "pk", "bv", "bs"]
    assert got.sorted_rows() == want.sorted_rows()


@pytest.mark.parametrize("build_n,probe_n,dup", [(1000, 50_000, 1), (6000, 400_000, 3), (300_000, 1_200_000, 2)])
def test_join_fixed_width_outputs_fused_probe(gpu, build_n, probe_n, dup):
    # only fixed-width outputs: the probe materialises them in one kernel
    # (staged per warp, one cursor atomic per run), repeated build keys
    # included
    rng = np.random.default_rng(build_n + probe_n + dup)
    bkeys = np.repeat(np.arange(build_n // dup, dtype=np.int64), dup)[:build_n]
    build = Table([Column("pk", "int32", bkeys), Column("bv", "int64", rng.integers(0, 10**9, len(bkeys)))])
    probe = Table([Column("fk", "int32", rng.integers(-5, build_n // dup + 5, probe_n)),
                   Column("pv", "int32", rng.integers(0, 100, probe_n))])
    j = ops.HashJoin("pk", "fk")
    j.put_build(build)
    j.finalize_build()
    got = j.probe(DeviceTable.from_host(probe))
    want = oops.hash_join(build, probe, "pk", "fk")
    assert got.names == want.names == ["fk", "pv", "pk", "bv"]
    assert got.num_rows == want.num_rows
    assert got.sorted_rows() == want.sorted_rows()


def test_join_int64_keys_and_multiple_build_batches(gpu):
    rng = np.random.default_rng(5)
    b1 = Table([Column("k", "int64", rng.integers(-2**40, 2**40, 3000)), Column("x", "int32", np.arange(3000))])
    b2 = Table([Column("k", "int64", b1["k"][:500] + 1), Column("x", "int32", np.arange(500))])
    probe = Table([Column("pk", "int64", np.concatenate([b1["k"], b2["k"], rng.integers(-2**40, 2**40, 3000)]))])
    j = ops.HashJoin("k", "pk", needed=["pk", "x"])
    j.put_build(b1)
    j.put_build(b2)
    j.finalize_build()
    got = j.probe(probe)
    b = Table([Column("k", "int64", np.concatenate([b1["k"], b2["k"]])),
               Column("x", "int32", np.concatenate([b1["x"], b2["x"]]))])
    want = oops.hash_join(b, probe, "k", "pk", ["pk", "x"])
    assert got.sorted_rows() == want.sorted_rows()


AGGS = [
    {"function": "SUM", "name": "s", "expr": times(col("v"), col("w"))},
    {"function": "COUNT", "name": "c"},
    {"function": "MIN", "name": "mn", "expr": col("w")},
    {"function": "MAX", "name": "mx", "expr": col("v")},
    {"function": "SUM", "name": "s32", "expr": col("w")},
]


@pytest.mark.parametrize("n,groups,hint", [(0, 1, 0), (1, 1, 0), (10_000, 5, 0), (100_000, 175, 256),
                                           (300_000, 50_000, 0), (300_000, 200_000, 400_000)])
def test_group_parity(gpu, n, groups, hint):
    rng = np.random.default_rng(n + groups)
    t = Table([Column("g", "int32", rng.integers(0, groups, n)), Column("v", "int64", rng.integers(-10**15, 10**15, n)),
               Column("w", "int32", rng.integers(-1000, 1000, n))])
    g = ops.Group(["g"], AGGS, hint)
    g.group(t)
    got = g.finalise()
    want = oops.group_by(t, ["g"], AGGS)
    assert got.names == want.names
    assert got.sorted_rows() == want.sorted_rows()


def test_group_sketch_sized_table_two_batches(gpu):
    # Batches large enough that the table is sized from a distinct-key sketch
    # rather than the row count; the second batch overlaps the first's keys
    # and re-sizes from the exact group count plus its own sketch.
    rng = np.random.default_rng(77)
    n = 2_200_000
    parts = [Table([Column("g", "int64", rng.integers(lo, lo + 1_000_000, n) * 7919),
                    Column("v", "int64", rng.integers(-10**12, 10**12, n))]) for lo in (0, 500_000)]
    aggs = [{"function": "SUM", "name": "s", "expr": col("v")}, {"function": "COUNT", "name": "c"}]
    g = ops.Group(["g"], aggs)
    for p in parts:
        g.group(DeviceTable.from_host(p))
    got = g.finalise()
    allt = Table([Column(c, "int64", np.concatenate([p[c] for p in parts])) for c in ("g", "v")])
    want = oops.group_by(allt, ["g"], aggs)
    assert got.num_rows == want.num_rows
    assert got.sorted_rows() == want.sorted_rows()


def test_group_sketch_sized_table_two_int32_keys(gpu):
    # two int32 key columns packed into one 64-bit key, a batch large enough
    # for the sketch-sized table, with MIN / MAX accumulators (which need the
    # table's init kernel rather than pre-filled memory)
    rng = np.random.default_rng(78)
    n = 2_300_000
    t = Table([Column("a", "int32", rng.integers(-700, 700, n)), Column("b", "int32", rng.integers(0, 1500, n)),
               Column("v", "int64", rng.integers(-10**9, 10**9, n))])
    aggs = [{"function": "SUM", "name": "s", "expr": col("v")}, {"function": "MIN", "name": "mn", "expr": col("v")},
            {"function": "MAX", "name": "mx", "expr": col("v")}, {"function": "COUNT", "name": "c"}]
    g = ops.Group(["a", "b"], aggs)
    g.group(DeviceTable.from_host(t))
    got = g.finalise()
    want = oops.group_by(t, ["a", "b"], aggs)
    assert got.num_rows == want.num_rows
    assert got.sorted_rows() == want.sorted_rows()


def test_group_two_keys_utf8_key_and_batches(gpu):
    rng = np.random.default_rng(9)
    parts = []
    for b in range(3):
        n = 20_000 + b
        parts.append(Table([Column("r", "utf8", [workloads.REGIONS[x] for x in rng.integers(0, 5, n)]),
                            Column("a", "int32", rng.integers(0, 25, n)),
                            Column("b", "int32", rng.integers(-3, 4, n)),
                            Column("v", "int64", rng.integers(0, 10**7, n))]))
    aggs = [{"function": "SUM", "name": "s", "expr": col("v")}, {"function": "COUNT", "name": "c"},
            {"function": "AVG", "name": "avg", "expr": col("v")}]
    g2 = ops.Group(["a", "b"], aggs)
    gs = ops.Group(["r"], aggs)
    for p in parts:
        g2.group(p)
        gs.group(DeviceTable.from_host(p))
    allt = Table([Column(c.name, c.type, np.concatenate([p.column(c.name).values for p in parts])
                         if c.type != "utf8" else sum((p[c.name] for p in parts), []))
                  for c in parts[0].columns])
    for g, keys in ((g2, ["a", "b"]), (gs, ["r"])):
        got = g.finalise()
        want = oops.group_by(allt, keys, aggs)
        gr = sorted(got.rows())
        wr = sorted(want.rows())
        assert [r[:-1] for r in gr] == [r[:-1] for r in wr]
        assert np.allclose([r[-1] for r in gr], [r[-1] for r in wr], rtol=1e-12)


def test_group_special_key_and_int64_wrap(gpu):
    big = np.iinfo(np.int64).max
    t = Table([Column("g", "int64", [-1, -1, 0, 5, -1]), Column("v", "int64", [big, big, 1, 2, 3])])
    aggs = [{"function": "SUM", "name": "s", "expr": col("v")}, {"function": "COUNT", "name": "c"}]
    g = ops.Group(["g"], aggs)
    g.group(t)
    got = g.finalise()
    assert got.sorted_rows() == oops.group_by(t, ["g"], aggs).sorted_rows()


CSV_FIELDS = [("i", "int32"), ("l", "int64"), ("p", "decimal(15,2)"), ("dt", "date32"), ("s", "utf8")]


def csv_text(n, seed=0, crlf=False, header=True, trailing=True):
    rng = np.random.default_rng(seed)
    lines = ["i|l|p|dt|s"] if header else []
    for r in range(n):
        cents = int(rng.integers(0, 10_000_000))
        frac = ["", ".5", f".{cents % 100:02d}"][r % 3]
        y, m, d = 1992 + r % 7, 1 + r % 12, 1 + r % 28
        s = "".join(chr(65 + int(x)) for x in rng.integers(0, 26, r % 11))
        if r % 5 == 0:
            s = f'"{s}"'
        lines.append(f"{int(rng.integers(-2**31, 2**31))}|{int(rng.integers(-2**62, 2**62))}|"
                     f"{'-' if r % 4 == 0 else ''}{cents // 100}{frac}|{y:04d}-{m:02d}-{d:02d}|{s}")
    text = ("\r\n" if crlf else "\n").join(lines)
    if trailing:
        text += "\r\n" if crlf else "\n"
    return text.encode()


@pytest.mark.parametrize("n,crlf,trailing", [(0, False, True), (1, False, False), (1000, True, True),
                                             (50_000, False, True), (50_001, False, False)])
def test_csv_parity(gpu, n, crlf, trailing):
    text = csv_text(n, seed=n, crlf=crlf, trailing=trailing)
    got = ops.csv_read(text, CSV_FIELDS, delimiter="|", has_header=True)
    want = oops.csv_parse(text, CSV_FIELDS, delimiter="|", has_header=True)
    assert got.names == want.names
    assert got.rows() == want.rows()


def test_csv_projection_and_malformed(gpu):
    text = csv_text(3000, seed=2)
    got = ops.csv_read(text, CSV_FIELDS, columns=["s", "p"], delimiter="|", has_header=True)
    want = oops.csv_parse(text, CSV_FIELDS, columns=["s", "p"], delimiter="|", has_header=True)
    assert got.rows() == want.rows()
    from flexpushdowndb_gb300 import GfpdbError

    with pytest.raises(GfpdbError) as ei:
        ops.csv_read(b"1|2|x|1992-01-01|a\n", CSV_FIELDS, delimiter="|")
    assert "malformed" in ei.value.message
    with pytest.raises(GfpdbError):
        ops.csv_read(b"1|2|3\n", CSV_FIELDS, delimiter="|")


def test_error_reporting_leaves_device_usable(gpu):
    from flexpushdowndb_gb300 import GfpdbError

    t = Table([Column("a", "int32", [1, 2, 0]), Column("b", "int32", [1, 0, 3])])
    with pytest.raises(GfpdbError) as ei:
        ops.Filter(eq(divide(col("a"), col("b")), num_lit(1)), t).evaluate(t)
    assert ei.value.code == 3  # device error word: integer divide by zero
    ok = ops.Filter(gt(col("a"), num_lit(0)), t).evaluate(t)
    assert ok.rows() == [(1, 1), (2, 0)]


def _probe_case(fact_rows, key_type, seed):
    tabs = workloads.star_tables(fact_rows=fact_rows, seed=seed)
    fact = tabs["fact"]
    if key_type == "int64":
        fact = Table([Column(c.name, "int64" if c.name.startswith("fk") else c.type, c.values) for c in fact.columns])
    blooms, seq = [], fact
    for i, c in ((2, 3), (3, 2), (4, 5), (1, 1)):
        d = oops.filter_table(tabs[f"d{i}"], eq(col(f"d{i}_f"), num_lit(c)))
        blooms.append((ops.BloomFilter([d], f"d{i}_pk"), f"fk{i}"))
        seq = oops.bloom_use(seq, oops.bloom_words(d[f"d{i}_pk"]), f"fk{i}")
    return fact, blooms, seq


@pytest.mark.parametrize("fact_rows,key_type,n_probes", [(1 << 20, "int32", 4), ((1 << 20) + 13, "int32", 1),
                                                         (3_000_001, "int64", 4), (2_500_007, "int32", 2)])
def test_select_probe_pipeline_large(gpu, fact_rows, key_type, n_probes):
    """Inputs of a million rows and more take the two-pass probe-only
    kernels (warp slices of 256 rows); output rows and their order match the
    oracle's sequential bloom uses, including a ragged last slice."""
    fact, blooms, _ = _probe_case(fact_rows, key_type, 2100 + n_probes)
    want = fact
    for bf, c in blooms[:n_probes]:
        want = oops.bloom_use(want, bf.words(), c)
    got = ops.select(DeviceTable.from_host(fact), None, blooms[:n_probes])
    assert got.num_rows == want.num_rows
    assert got.rows() == want.rows()


def test_select_probe_pipeline_unaligned_columns(gpu):
    """Key columns that do not start on a 16-byte boundary are read with
    scalar loads; results are the same."""
    import torch

    fact, blooms, seq = _probe_case((1 << 20) + 5, "int32", 2200)
    dt = DeviceTable.from_host(fact)
    shifted = []
    for ts in dt.tensors:
        views = []
        for t in ts:
            buf = torch.empty(t.numel() + 1, dtype=t.dtype, device=t.device)
            buf[1:] = t
            views.append(buf[1:])
        shifted.append(views)
    got = ops.select(DeviceTable(dt.names, dt.types, shifted, dt.num_rows), None, blooms)
    assert got.rows() == seq.rows()


def test_csv_lineitem_exact_values(gpu):
    """The lineitem text (fields up to 40 bytes, rows crossing 64-byte thread
    chunks and 16 KiB tiles) parses into exactly the values it was written
    from, every column."""
    rows = 120_000
    text = workloads.lineitem_csv(rows, seed=3300)
    got = ops.csv_read(text, workloads.LINEITEM_FIELDS, delimiter="|")
    want = workloads.lineitem_columns(rows, seed=3300)
    assert got.num_rows == rows
    for name, ty in workloads.LINEITEM_FIELDS:
        if ty == "utf8":
            lens, chars = want[name]
            offs, data = got.column(name).values
            assert np.array_equal(np.diff(offs), lens), name
            assert np.array_equal(data, chars), name
        else:
            assert np.array_equal(np.asarray(got[name], dtype=np.int64), want[name]), name


def test_csv_long_fields_span_tiles(gpu):
    """Fields longer than a thread's 64 bytes and a tile's 16 KiB."""
    rng = np.random.default_rng(3400)
    lines, vals = [], []
    for r in range(50):
        s = "x" * int(rng.integers(0, 40_000))
        lines.append(f"{r}|{s}|{-r * 7}")
        vals.append((r, s, -r * 7))
    text = ("\n".join(lines) + "\n").encode()
    got = ops.csv_read(text, [("a", "int32"), ("s", "utf8"), ("b", "int64")], delimiter="|")
    assert got.rows() == vals


def test_csv_malformed_row_in_large_text(gpu):
    from flexpushdowndb_gb300 import GfpdbError

    text = bytearray(workloads.lineitem_csv(20_000, seed=3500))
    # an extra field in row 12,345 (and one fewer in the next row: the
    # separator total stays a multiple of the field count)
    nl = [i for i, c in enumerate(text) if c == 10]
    text[nl[12_344] - 1 : nl[12_344] - 1] = b"|"
    end = nl[12_345] + 1
    cut = text.index(b"|", end)
    del text[cut]
    with pytest.raises(GfpdbError) as ei:
        ops.csv_read(bytes(text), workloads.LINEITEM_FIELDS, delimiter="|")
    assert "malformed" in ei.value.message
    with pytest.raises(GfpdbError):
        ops.csv_read(b"1|2\n3\n", [("a", "int32"), ("b", "int32")], delimiter="|")


def test_csv_empty_and_utf8_only(gpu):
    got = ops.csv_read(b"", [("a", "int32")], delimiter="|")
    assert got.num_rows == 0
    got = ops.csv_read(b"||\n|x|\n", [("a", "utf8"), ("b", "utf8"), ("c", "utf8")], delimiter="|")
    assert got.rows() == [("", "", ""), ("", "x", "")]


def test_csv_dense_and_sparse_tiles(gpu):
    """Tiles with more separators than a tile stages in shared memory (fields
    of one or two bytes) next to tiles of long fields; empty fields, quotes
    and CRLF in both."""
    rng = np.random.default_rng(3600)
    fields = [("a", "int32"), ("b", "int64"), ("s", "utf8")]
    lines = ["a|b|s"]
    for blk in range(12):
        if blk % 2 == 0:
            for r in range(int(rng.integers(2000, 9000))):
                lines.append(f"{r % 10}|{r % 7}|{'' if r % 3 else chr(97 + r % 26)}")
        else:
            for r in range(int(rng.integers(100, 600))):
                s = "".join(chr(65 + int(x)) for x in rng.integers(0, 26, int(rng.integers(0, 90))))
                lines.append(f"{int(rng.integers(-2**31, 2**31))}|{int(rng.integers(-2**62, 2**62))}|"
                             f"{chr(34) + s + chr(34) if r % 4 == 0 else s}")
    text = ("\r\n".join(lines) + "\r\n").encode()
    got = ops.csv_read(text, fields, delimiter="|", has_header=True)
    want = oops.csv_parse(text, fields, delimiter="|", has_header=True)
    assert got.num_rows == len(lines) - 1
    assert got.rows() == want.rows()
    got = ops.csv_read(text, fields, columns=["s", "a"], delimiter="|", has_header=True)
    assert got.rows() == oops.csv_parse(text, fields, columns=["s", "a"], delimiter="|", has_header=True).rows()

    from flexpushdowndb_gb300 import GfpdbError

    bad = bytearray(text)
    cut = len(lines[0]) + 2 + 6 * 1000  # inside the first dense block: "x|y|" at a row's start
    row_start = bad.index(b"\n", cut) + 1
    bad[row_start:row_start + 1] = b"x"  # an int32 field that is not a number
    with pytest.raises(GfpdbError) as ei:
        ops.csv_read(bytes(bad), fields, delimiter="|", has_header=True)
    assert "malformed" in ei.value.message


LITE_PREDICATES = [
    gt(num_lit(5), col("k")),  # literal on the left
    lte(num_lit(-3, "int64"), col("i64")),
    and_(gte(col("d"), num_lit(9000, "date32")), neq(col("k"), num_lit(4)), lte(col("i32"), num_lit(0))),
    or_(*[eq(col("k"), num_lit(v)) for v in range(8)]),  # eight leaves in one clause
    or_(*[eq(col("k"), num_lit(v)) for v in range(9)]),  # nine: beyond the compact kernel's leaves
    and_(or_(lt(col("i32"), num_lit(-500)), gt(col("i64"), num_lit(0, "int64"))), eq(col("k"), num_lit(1))),
]


@pytest.mark.parametrize("pi", range(len(LITE_PREDICATES)))
@pytest.mark.parametrize("n", [3, 1023, 1024, 1025, 262_143, 262_144, 262_145])
def test_filter_small_input_shapes(gpu, pi, n):
    """Inputs up to 2^18 rows with integer column-vs-literal predicates (the
    compact selection kernel) and just past it (the general kernel), at tile
    edges, with utf8 and float outputs moved as well."""
    t = rand_table(n, seed=7 * n + pi)
    pred = LITE_PREDICATES[pi]
    got = ops.Filter(pred, t).evaluate(t)
    assert got.rows() == oops.filter_table(t, pred).rows()


@pytest.mark.parametrize("n", [1, 777, 4096, 200_000])
def test_small_select_with_probes_and_predicate(gpu, n):
    """Bloom probes on int32 and int64 keys together with a predicate, over
    small inputs."""
    rng = np.random.default_rng(n)
    t = Table([Column("a", "int32", rng.integers(0, 5000, n)), Column("b", "int64", rng.integers(-10**9, 10**9, n)),
               Column("c", "int32", rng.integers(0, 100, n)), Column("s", "utf8", [f"v{x}" for x in range(n)])])
    ka = rng.choice(5000, 700, replace=False).astype(np.int64)
    kb = np.asarray(t["b"], dtype=np.int64)[rng.random(n) < 0.5]
    ta = Table([Column("a", "int32", ka)])
    tb = Table([Column("b", "int64", kb)])
    blooms = [(ops.BloomFilter([ta], "a"), "a"), (ops.BloomFilter([tb], "b", 12, 4), "b")]
    pred = and_(lt(col("c"), num_lit(60)), neq(col("c"), num_lit(7)))
    got = ops.select(DeviceTable.from_host(t), ops.Filter(pred, t), blooms)
    want = oops.bloom_use(oops.bloom_use(oops.filter_table(t, pred), oops.bloom_words(ka), "a"),
                          oops.bloom_words(kb, 12, 4), "b", 4)
    assert got.rows() == want.rows()


def test_join_info_after_build(gpu):
    """Build-side statistics: rows, table capacity (power of two at load
    factor 0.5) and the longest probe run the build recorded."""
    keys = np.arange(10_000, dtype=np.int64) * 3
    build = Table([Column("pk", "int32", keys), Column("v", "int32", np.arange(10_000))])
    j = ops.HashJoin("pk", "fk")
    j.put_build(build)
    j.finalize_build()
    info = j.info()
    assert info["build_rows"] == 10_000
    assert info["capacity"] == 32_768
    assert 0 <= info["max_probe"] < 64  # linear probing at load 0.31


def test_select_probe_first_filter_in_global_memory(gpu):
    """A first filter too large for shared memory (200,000 keys at 16 bits
    per key) is probed through L1/L2; results match the oracle."""
    fact, _, _ = _probe_case(1_200_000, "int32", 2300)
    tabs = workloads.star_tables(fact_rows=10, seed=2300)
    big = tabs["d2"]
    bf = ops.BloomFilter([big], "d2_pk", 16, 3)
    assert bf.info()["num_blocks"] * 32 > 96 * 1024
    d3 = oops.filter_table(tabs["d3"], eq(col("d3_f"), num_lit(2)))
    blooms = [(bf, "fk2"), (ops.BloomFilter([d3], "d3_pk"), "fk3")]
    want = oops.bloom_use(oops.bloom_use(fact, bf.words(), "fk2"), oops.bloom_words(d3["d3_pk"]), "fk3")
    got = ops.select(DeviceTable.from_host(fact), None, blooms)
    assert got.rows() == want.rows()


@pytest.mark.parametrize("pi", [0, 2, 3, 5])
def test_filter_large_simple_predicates(gpu, pi):
    """A million rows and more with an integer column-vs-literal predicate
    take the two-pass kernels (warp slices, then the gather), utf8 and float
    outputs included; rows and order match the oracle."""
    n = (1 << 20) + 4097
    t = rand_table(n, seed=300 + pi)
    pred = LITE_PREDICATES[pi]
    got = ops.Filter(pred, t).evaluate(DeviceTable.from_host(t))
    assert got.rows() == oops.filter_table(t, pred).rows()


def test_select_large_predicate_with_probes(gpu):
    """A predicate and a chain of bloom probes over 1.2 million rows in one
    two-pass selection."""
    fact, blooms, seq = _probe_case(1_200_003, "int32", 2400)
    pred = and_(gt(col("qty"), num_lit(10)), lte(num_lit(3), col("discount")))
    got = ops.select(DeviceTable.from_host(fact), ops.Filter(pred, fact), blooms)
    assert got.rows() == oops.filter_table(seq, pred).rows()


def test_group_and_join_clear(gpu):
    """clear() (GroupAbstractKernel.h:44, HashJoinArrowKernel.h:56): a
    cleared group-by starts over with the same spec, a cleared join takes a
    new build side."""
    from flexpushdowndb_gb300.expression import col as c_
    from flexpushdowndb_gb300.ops import aggregate

    rng = np.random.default_rng(31)
    t1 = Table([Column("k", "int32", rng.integers(0, 50, 5000)), Column("v", "int64", rng.integers(0, 100, 5000))])
    t2 = Table([Column("k", "int32", rng.integers(0, 9, 700)), Column("v", "int64", rng.integers(0, 100, 700))])
    g = ops.Group(["k"], [aggregate("SUM", "s", c_("v")), aggregate("COUNT", "n")])
    g.group(DeviceTable.from_host(t1))
    g.clear()
    g.group(DeviceTable.from_host(t2))
    want = oops.group_by(t2, ["k"], [{"function": "SUM", "name": "s", "expr": c_("v")},
                                     {"function": "COUNT", "name": "n"}])
    assert g.finalise().sorted_rows() == want.sorted_rows()
    b1 = Table([Column("bk", "int32", np.arange(100)), Column("bv", "int64", np.arange(100) * 3)])
    b2 = Table([Column("bk", "int32", np.arange(50, 60)), Column("bv", "int64", np.arange(10) * 7)])
    probe = Table([Column("pk", "int32", rng.integers(0, 120, 2000))])
    j = ops.HashJoin("bk", "pk")
    j.put_build(DeviceTable.from_host(b1))
    j.finalize_build()
    j.probe(DeviceTable.from_host(probe))
    j.clear()
    j.put_build(DeviceTable.from_host(b2))
    j.finalize_build()
    got = j.probe(DeviceTable.from_host(probe))
    assert got.sorted_rows() == oops.hash_join(b2, probe, "bk", "pk").sorted_rows()


def _two_key_tables(seed, n_build=3000, n_probe=40_000, utf8=False, wide=False):
    rng = np.random.default_rng(seed)
    words = [f"k{i}" for i in range(13)]
    bk1 = rng.integers(0, 60, n_build)
    bk2 = rng.integers(0, 70, n_build)
    build = [Column("b1", "int64" if wide else "int32", bk1 * (10**10 if wide else 1)),
             Column("b2", "int32", bk2), Column("bv", "int64", rng.integers(0, 10**9, n_build))]
    probe = [Column("p1", "int64" if wide else "int32", rng.integers(0, 66, n_probe) * (10**10 if wide else 1)),
             Column("p2", "int32", rng.integers(0, 75, n_probe)), Column("pv", "int32", np.arange(n_probe))]
    if utf8:
        build.append(Column("bs", "utf8", [words[i] for i in rng.integers(0, 13, n_build)]))
        probe.append(Column("ps", "utf8", [words[i] for i in rng.integers(0, 13, n_probe)]))
    return Table(build), Table(probe)


@pytest.mark.parametrize("utf8,wide", [(False, False), (True, False), (False, True)])
def test_two_key_join_matches_oracle(gpu, utf8, wide):
    """Joins on two (or three, with a utf8 column) key columns: repeated keys
    on both sides, int64 keys with values past 32 bits, utf8 keys; every pair
    of rows whose key columns are equal, and no other (HashJoinPredicate.h:25-26)."""
    build, probe = _two_key_tables(77 + utf8 + 2 * wide, utf8=utf8, wide=wide)
    bk, pk = ["b1", "b2"] + (["bs"] if utf8 else []), ["p1", "p2"] + (["ps"] if utf8 else [])
    needed = ["pv", "p1", "bv", "b2"] + (["ps"] if utf8 else [])
    j = ops.HashJoin(bk, pk, needed)
    j.put_build(DeviceTable.from_host(build))
    j.finalize_build()
    got = j.probe(DeviceTable.from_host(probe))
    want = oops.hash_join_keys(build, probe, bk, pk, needed)
    assert got.names == want.names
    assert got.sorted_rows() == want.sorted_rows()


def test_two_key_bloom_filter(gpu):
    """A bloom filter over two key columns: every probe row whose key pair is
    in the build side passes (no false negatives); few others do."""
    build, probe = _two_key_tables(91, n_build=2000, n_probe=100_000)
    bf = ops.BloomFilter([build], ["b1", "b2"])
    kept = bf.use(DeviceTable.from_host(probe), ["p1", "p2"])
    inside = set(zip(build["b1"].tolist(), build["b2"].tolist()))
    pairs = list(zip(probe["p1"].tolist(), probe["p2"].tolist()))
    want_rows = {r for r, k in enumerate(pairs) if k in inside}
    kept_rows = set(kept["pv"].tolist())
    assert want_rows <= kept_rows
    assert len(kept_rows - want_rows) / max(1, len(pairs) - len(want_rows)) < 0.035
    with pytest.raises(GfpdbError):
        bf.use(DeviceTable.from_host(probe), "p1")  # built over two columns


def test_two_key_join_in_a_plan(gpu):
    from flexpushdowndb_gb300 import plan

    build, probe = _two_key_tables(93)
    p = plan.Plan()
    p.scan("sb", "b")
    p.scan("sp", "p")
    p._add({"type": "HashJoinArrowPOp", "name": "j", "buildProducers": ["sb"], "probeProducers": ["sp"],
            "buildKeys": ["b1", "b2"], "probeKeys": ["p1", "p2"], "projectColumnNames": ["pv", "bv"]})
    p.connect("sb", "j")
    p.connect("sp", "j")
    p.collate("c", "j")
    got = plan.execute(p, {"b": build, "p": probe}).table
    want = oops.hash_join_keys(build, probe, ["b1", "b2"], ["p1", "p2"], ["pv", "bv"])
    assert got.sorted_rows() == want.sorted_rows()
