"""Seeded synthetic workloads and their plans.

Inputs come from SplitMix64 (Steele, Lea, Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014) evaluated counter-style, so
any column of any partition can be regenerated from (seed, index) alone.
Seeds: config id * 1000 + partition, plus a per-column stream number.

Workloads (shapes of the reference's evaluation, all synthetic):
  two_table  - fact 1,000,000 x {fk, qty, price_cents}; dim 20,000 x
               {pk, category, region}; filter category < 5, join fk = pk,
               group by region -> sum(price_cents * qty), count(*).
  star       - SSB-SF1-shaped star: fact 6,000,000 x {fk1..fk4, qty,
               price_cents, discount}; dims of 30,000 / 200,000 / 2,000 /
               2,556 rows x {pk, f, g}; dim filters f = const keeping 1/5,
               1/25, 1/7, 1/7; forward + backward bloom predicate transfer,
               4-way join, group by (d2_g, d4_g) (~175 groups) ->
               sum(price*qty), sum(price*discount), count(*).
"""

from __future__ import annotations

import numpy as np

from .expression import and_, col, eq, gte, lt, lte, num_lit, times
from .ops import aggregate
from .plan import Plan
from .tupleset import Column, Table

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, start: int = 0) -> np.ndarray:
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int, lo: int, hi: int, start: int = 0) -> np.ndarray:
    """Integers uniform on [lo, hi] (inclusive), as int64."""
    r = splitmix64(seed * 1_000_003 + stream, n, start)
    span = np.uint64(hi - lo + 1)
    return (r % span).astype(np.int64) + lo


REGIONS = ["AFRICA  ", "AMERICA ", "ASIA    ", "EUROPE  ", "MIDEAST "]


# ------------------------------------------------------------------ two-table


def two_table_tables(fact_rows: int = 1_000_000, dim_rows: int = 20_000, seed: int = 1000) -> dict[str, Table]:
    fk = uniform(seed, 1, fact_rows, 1, dim_rows)
    qty = uniform(seed, 2, fact_rows, 1, 50)
    price = uniform(seed, 3, fact_rows, 90_000, 10_500_000)
    pk = np.arange(1, dim_rows + 1, dtype=np.int64)
    cat = uniform(seed, 4, dim_rows, 0, 24)
    reg = uniform(seed, 5, dim_rows, 0, len(REGIONS) - 1)
    fact = Table([Column("fk", "int32", fk), Column("qty", "int32", qty), Column("price_cents", "int64", price)])
    dim = Table([Column("pk", "int32", pk), Column("category", "int32", cat),
                 Column("region", "utf8", [REGIONS[i] for i in reg])])
    return {"fact": fact, "dim": dim}


def two_table_plan(category_lt: int = 5, chunk_rows: int = 0) -> Plan:
    p = Plan()
    p.scan("scan_dim", "dim", ["pk", "category", "region"])
    p.filter("filter_dim", "scan_dim", lt(col("category"), num_lit(category_lt, "int32")), ["pk", "region"])
    p.scan("scan_fact", "fact", ["fk", "qty", "price_cents"], chunk_rows=chunk_rows)
    p.hash_join("join", "filter_dim", "scan_fact", "pk", "fk", ["region", "qty", "price_cents"])
    p.group("group", "join", ["region"],
            [aggregate("SUM", "revenue", times(col("price_cents"), col("qty"))), aggregate("COUNT", "cnt")],
            groups_hint=8)
    p.collate("collate", "group")
    return p


# ----------------------------------------------------------------------- star

STAR_DIM_ROWS = (30_000, 200_000, 2_000, 2_556)
STAR_FILTER_VALUES = (5, 25, 7, 7)   # f uniform over this many values
STAR_GROUP_VALUES = (10, 25, 10, 7)  # g uniform over this many values (d2_g x d4_g = 175 groups)
STAR_DEFAULT_CONSTS = (1, 3, 2, 5)   # dim filter: f == const


def star_dims(seed: int = 2000) -> dict[str, Table]:
    out = {}
    for i, n in enumerate(STAR_DIM_ROWS, start=1):
        out[f"d{i}"] = Table([
            Column(f"d{i}_pk", "int32", np.arange(1, n + 1, dtype=np.int64)),
            Column(f"d{i}_f", "int32", uniform(seed, 10 + i, n, 0, STAR_FILTER_VALUES[i - 1] - 1)),
            Column(f"d{i}_g", "int32", uniform(seed, 20 + i, n, 0, STAR_GROUP_VALUES[i - 1] - 1)),
        ])
    return out


def star_fact(rows: int = 6_000_000, seed: int = 2000, start: int = 0) -> Table:
    cols = [Column(f"fk{i}", "int32", uniform(seed, i, rows, 1, n, start)) for i, n in enumerate(STAR_DIM_ROWS, 1)]
    cols += [
        Column("qty", "int32", uniform(seed, 5, rows, 1, 50, start)),
        Column("price_cents", "int64", uniform(seed, 6, rows, 90_000, 10_500_000, start)),
        Column("discount", "int32", uniform(seed, 7, rows, 0, 10, start)),
    ]
    return Table(cols)


def star_tables(fact_rows: int = 6_000_000, seed: int = 2000) -> dict[str, Table]:
    t = star_dims(seed)
    t["fact"] = star_fact(fact_rows, seed)
    return t


def star_plan(consts=STAR_DEFAULT_CONSTS, bits_per_key: int = 10, num_hashes: int = 3, chunk_rows: int = 0,
              backward: bool = True, ranges=None, fact_tables=("fact",), probe_order=(2, 3, 4, 1)) -> Plan:
    """Forward + backward bloom predicate transfer, then the 4-way join and
    group-by, in the shape SmallToLargePredTransOrder builds
    (fpdb-executor/src/physical/transform/pred-trans/SmallToLargePredTransOrder.cpp:38-214).
    Dimension filters are f == const, or lo <= f <= hi with `ranges`; the
    fact table may be several partitions, one scan each (the reference's one
    scan operator per partition, PrePToPTransformer.cpp:1078-1100)."""
    p = Plan()
    dim_tail = {}
    fwd = {}
    for i in range(1, 5):
        p.scan(f"scan_d{i}", f"d{i}", [f"d{i}_pk", f"d{i}_f", f"d{i}_g"])
        keep = [f"d{i}_pk", f"d{i}_g"] if i in (2, 4) else [f"d{i}_pk"]
        if ranges is not None:
            lo, hi = ranges[i - 1]
            pred = and_(gte(col(f"d{i}_f"), num_lit(int(lo), "int32")), lte(col(f"d{i}_f"), num_lit(int(hi), "int32")))
        else:
            pred = eq(col(f"d{i}_f"), num_lit(int(consts[i - 1]), "int32"))
        p.filter(f"filter_d{i}", f"scan_d{i}", pred, keep)
        fwd[i] = p.bloom_create(f"bf_fwd_create_d{i}", f"filter_d{i}", f"d{i}_pk", bits_per_key, num_hashes)
        dim_tail[i] = fwd[i]
    fact_cols = ["fk1", "fk2", "fk3", "fk4", "qty", "price_cents", "discount"]
    scans = [p.scan(f"scan_{t}", t, fact_cols, chunk_rows=chunk_rows) for t in fact_tables]
    # forward: the most selective filters first (1/25, 1/7, 1/7, 1/5)
    first = True
    tail = None
    for i in probe_order:
        name = f"bf_fwd_use_fk{i}"
        if first:
            tail = p.bloom_use(name, scans[0], fwd[i], f"fk{i}")
            for sc in scans[1:]:
                p.connect(sc, name)
            first = False
        else:
            tail = p.bloom_use(name, tail, fwd[i], f"fk{i}")
    if backward:
        for i in range(1, 5):
            c = p.bloom_create(f"bf_bwd_create_fk{i}", tail, f"fk{i}", bits_per_key, num_hashes)
            dim_tail[i] = p.bloom_use(f"bf_bwd_use_d{i}", dim_tail[i], c, f"d{i}_pk")
            tail = c
    fact_cols = ["fk1", "fk2", "fk3", "fk4", "qty", "price_cents", "discount"]
    carried: list[str] = []
    for i in range(1, 5):
        fact_cols = [c for c in fact_cols if c != f"fk{i}"]
        if i in (2, 4):
            carried.append(f"d{i}_g")
        tail = p.hash_join(f"join_d{i}", dim_tail[i], tail, f"d{i}_pk", f"fk{i}", fact_cols + carried)
    p.group("group", tail, ["d2_g", "d4_g"], [
        aggregate("SUM", "revenue", times(col("price_cents"), col("qty"))),
        aggregate("SUM", "discount_revenue", times(col("price_cents"), col("discount"))),
        aggregate("COUNT", "cnt"),
    ], groups_hint=256)
    p.collate("collate", "group")
    return p


def star_plan_planned(consts=STAR_DEFAULT_CONSTS, fact_rows: int = 6_000_000, bits_per_key: int = 10,
                      num_hashes: int = 3, ranges=None) -> Plan:
    """The star query with its bloom predicate transfer derived from the join
    graph by the planner (Plan.predicate_transfer, SmallToLargePredTransOrder)
    rather than written out: each dimension's filtered scan and the fact scan
    are the base tables (row counts, and the dimension filters' selectivity),
    the four fact-to-dimension joins the graph; the joins and the group-by
    then attach to each table's last operator."""
    p = Plan()
    tables = {}
    for i in range(1, 5):
        p.scan(f"scan_d{i}", f"d{i}", [f"d{i}_pk", f"d{i}_f", f"d{i}_g"])
        keep = [f"d{i}_pk", f"d{i}_g"] if i in (2, 4) else [f"d{i}_pk"]
        if ranges is not None:
            lo, hi = ranges[i - 1]
            pred = and_(gte(col(f"d{i}_f"), num_lit(int(lo), "int32")), lte(col(f"d{i}_f"), num_lit(int(hi), "int32")))
            sel = (hi - lo + 1) / STAR_FILTER_VALUES[i - 1]
        else:
            pred = eq(col(f"d{i}_f"), num_lit(int(consts[i - 1]), "int32"))
            sel = 1 / STAR_FILTER_VALUES[i - 1]
        p.filter(f"filter_d{i}", f"scan_d{i}", pred, keep)
        tables[f"filter_d{i}"] = (STAR_DIM_ROWS[i - 1], sel)
    fact_cols = ["fk1", "fk2", "fk3", "fk4", "qty", "price_cents", "discount"]
    p.scan("scan_fact", "fact", fact_cols)
    tables["scan_fact"] = (fact_rows, 1.0)
    joins = [{"left": "scan_fact", "right": f"filter_d{i}", "leftColumns": [f"fk{i}"], "rightColumns": [f"d{i}_pk"],
              "joinType": "INNER"} for i in range(1, 5)]
    out = p.predicate_transfer(tables, joins, bits_per_key, num_hashes)
    tail = out["scan_fact"]
    carried: list[str] = []
    for i in range(1, 5):
        fact_cols = [c for c in fact_cols if c != f"fk{i}"]
        if i in (2, 4):
            carried.append(f"d{i}_g")
        tail = p.hash_join(f"join_d{i}", out[f"filter_d{i}"], tail, f"d{i}_pk", f"fk{i}", fact_cols + carried)
    p.group("group", tail, ["d2_g", "d4_g"], [
        aggregate("SUM", "revenue", times(col("price_cents"), col("qty"))),
        aggregate("SUM", "discount_revenue", times(col("price_cents"), col("discount"))),
        aggregate("COUNT", "cnt"),
    ], groups_hint=256)
    p.collate("collate", "group")
    return p


# -------------------------------------------------------------------- batched
#
# The batched form: the star query's fact table split into partitions of
# uneven size, and query variants that differ in their dimension filter
# ranges. Dimension filter columns are uniform over 100 values so a variant
# selecting k values of a dimension has selectivity k% (1% to 40%).

BATCH_FILTER_VALUES = 100


BATCH_SEED = 4106  # 64 partitions of 59,952,713 rows in all


def batch_partition_sizes(n_parts: int = 64, lo: int = 50_000, hi: int = 4_000_000, seed: int = BATCH_SEED) -> list[int]:
    """Partition sizes log-uniform in [lo, hi]."""
    u = splitmix64(seed, n_parts).astype(np.float64) / float(2**64)
    return [int(round(np.exp(np.log(lo) + x * (np.log(hi) - np.log(lo))))) for x in u]


def batch_tables(n_parts: int = 64, sizes=None, seed: int = BATCH_SEED) -> dict[str, Table]:
    sizes = sizes or batch_partition_sizes(n_parts, seed=seed)
    out = {}
    for i, n in enumerate(STAR_DIM_ROWS, start=1):
        out[f"d{i}"] = Table([
            Column(f"d{i}_pk", "int32", np.arange(1, n + 1, dtype=np.int64)),
            Column(f"d{i}_f", "int32", uniform(seed, 10 + i, n, 0, BATCH_FILTER_VALUES - 1)),
            Column(f"d{i}_g", "int32", uniform(seed, 20 + i, n, 0, STAR_GROUP_VALUES[i - 1] - 1)),
        ])
    start = 0
    for p, n in enumerate(sizes):
        out[f"p{p}"] = star_fact(n, seed=seed, start=start)
        start += n
    return out


def batch_queries(n_queries: int = 32, seed: int = 4100) -> list[list[tuple[int, int]]]:
    """Per query and dimension a range [0, k - 1] with k in [1, 40]."""
    k = uniform(seed, 1, n_queries * 4, 1, 40).reshape(n_queries, 4)
    return [[(0, int(k[q, d]) - 1) for d in range(4)] for q in range(n_queries)]


def star_batch_spec(fact_tables, queries, load_factor: float = 0.5, items_per_thread: int = 2,
                    blocks_per_sm: int = 4, probe_order=None, groups_hint: int = 256) -> dict:
    """probe_order None lets the engine order the dimensions (shared-memory
    staged ones first, then by size)."""
    spec = {
        "factTables": list(fact_tables),
        "dimensions": [{"table": f"d{i}", "key": f"d{i}_pk", "factKey": f"fk{i}", "filterColumn": f"d{i}_f"}
                       for i in range(1, 5)],
        "groupBy": [{"dimension": 1, "column": "d2_g"}, {"dimension": 3, "column": "d4_g"}],
        "aggregates": [{"function": "SUM", "name": "revenue", "columns": ["price_cents", "qty"]},
                       {"function": "SUM", "name": "discount_revenue", "columns": ["price_cents", "discount"]},
                       {"function": "COUNT", "name": "cnt"}],
        "queries": [[list(r) for r in q] for q in queries],
        "loadFactor": load_factor,
        "itemsPerThread": items_per_thread,
        "blocksPerSm": blocks_per_sm,
        "groupsHint": groups_hint,
    }
    if probe_order is not None:
        spec["probeOrder"] = list(probe_order)
    return spec


# ------------------------------------------------------------------------ CSV
#
# TPC-H-lineitem-shaped '|'-delimited text: per row 4 int32 uniform on
# [1, 2^20], 4 decimal(15,2) uniform on [0, 100000.00] written with two
# fractional digits, 2 dates uniform on 1992-01-01..1998-12-31 as YYYY-MM-DD,
# and 6 strings of length uniform on [10, 40] over [A-Za-z0-9 ]. Generated
# with vectorised digit writes, in chunks of rows, from SplitMix64 streams.

LINEITEM_FIELDS = ([(f"i{k}", "int32") for k in range(1, 5)] + [(f"d{k}", "decimal(15,2)") for k in range(1, 5)]
                   + [("t1", "date32"), ("t2", "date32")] + [(f"s{k}", "utf8") for k in range(1, 7)])
CSV_SEED = 3000
_ALPHABET = np.frombuffer(b"ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789 ", dtype=np.uint8)
DATE_LO = 8035   # 1992-01-01 as days since 1970-01-01
DATE_HI = 10591  # 1998-12-31


def civil_from_days(z: np.ndarray):
    """(year, month, day) of days since 1970-01-01 (H. Hinnant's
    civil_from_days, vectorised)."""
    z = z.astype(np.int64) + 719468
    era = np.floor_divide(z, 146097)
    doe = z - era * 146097
    yoe = (doe - doe // 1460 + doe // 36524 - doe // 146096) // 365
    y = yoe + era * 400
    doy = doe - (365 * yoe + yoe // 4 - yoe // 100)
    mp = (5 * doy + 2) // 153
    d = doy - (153 * mp + 2) // 5 + 1
    m = np.where(mp < 10, mp + 3, mp - 9)
    return y + (m <= 2), m, d


def _ndigits(x: np.ndarray) -> np.ndarray:
    n = np.ones(x.shape, dtype=np.int64)
    for k in range(1, 19):
        n += x >= 10**k
    return n


def _put_uint(buf: np.ndarray, pos: np.ndarray, x: np.ndarray, nd: np.ndarray) -> None:
    x = x.astype(np.int64)
    for k in range(int(nd.max()) if len(nd) else 0):
        m = nd > k
        buf[pos[m] + nd[m] - 1 - k] = 48 + (x[m] // 10**k) % 10


def lineitem_columns(rows: int, seed: int = CSV_SEED, start: int = 0) -> dict[str, np.ndarray]:
    """The typed values of rows [start, start + rows) (int32 as int64, decimals
    in cents, dates in days since the epoch; strings as (lengths, chars))."""
    cols = {}
    for k in range(1, 5):
        cols[f"i{k}"] = uniform(seed, k, rows, 1, 1 << 20, start)
    for k in range(1, 5):
        cols[f"d{k}"] = uniform(seed, 4 + k, rows, 0, 10_000_000, start)
    cols["t1"] = uniform(seed, 9, rows, DATE_LO, DATE_HI, start)
    cols["t2"] = uniform(seed, 10, rows, DATE_LO, DATE_HI, start)
    for k in range(1, 7):
        lens = uniform(seed, 10 + k, rows, 10, 40, start)
        # the chars of row r start at a counter position that does not depend
        # on the chunking: 40 slots per row
        pos = np.repeat((np.arange(rows, dtype=np.int64) + start) * 40, lens) + (
            np.arange(int(lens.sum()), dtype=np.int64) - np.repeat(np.cumsum(lens) - lens, lens))
        chars = _ALPHABET[_stream_at(seed * 1_000_003 + 20 + k, pos) % np.uint64(len(_ALPHABET))]
        cols[f"s{k}"] = (lens, chars)
    return cols


def _stream_at(seed: int, idx: np.ndarray) -> np.ndarray:
    """SplitMix64 outputs at arbitrary counter positions."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + (idx.astype(np.uint64) + np.uint64(1)) * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def lineitem_csv(rows: int, seed: int = CSV_SEED, chunk: int = 250_000, processes: int = 0) -> bytes:
    """The text of `rows` lineitem-shaped rows, '|'-delimited, '\\n'-terminated.
    Chunks are independent (counter-based streams); with processes > 1 they
    are generated by a pool of spawned processes (never forked: the caller
    may already hold a CUDA context)."""
    jobs = [(min(chunk, rows - start), seed, start) for start in range(0, rows, chunk)]
    if processes > 1 and len(jobs) > 1:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(min(processes, len(jobs))) as pool:
            return b"".join(pool.starmap(_lineitem_chunk, jobs))
    return b"".join(_lineitem_chunk(*j) for j in jobs)


def _lineitem_chunk(rows: int, seed: int, start: int) -> bytes:
    c = lineitem_columns(rows, seed, start)
    names = [n for n, _ in LINEITEM_FIELDS]
    lens = []
    for n, ty in LINEITEM_FIELDS:
        if ty == "int32":
            lens.append(_ndigits(c[n]))
        elif ty.startswith("decimal"):
            lens.append(_ndigits(c[n] // 100) + 3)
        elif ty == "date32":
            lens.append(np.full(rows, 10, dtype=np.int64))
        else:
            lens.append(c[n][0])
    L = np.stack(lens)                          # [field, row]
    row_len = L.sum(axis=0) + len(names)        # separators + newline
    row_off = np.cumsum(row_len) - row_len
    buf = np.empty(int(row_len.sum()), dtype=np.uint8)
    off = row_off.copy()
    for f, (n, ty) in enumerate(LINEITEM_FIELDS):
        ln = L[f]
        if ty == "int32":
            _put_uint(buf, off, c[n], ln)
        elif ty.startswith("decimal"):
            ip = c[n] // 100
            nd = ln - 3
            _put_uint(buf, off, ip, nd)
            buf[off + nd] = ord(".")
            _put_uint(buf, off + nd + 1, c[n] % 100, np.full(rows, 2, dtype=np.int64))
        elif ty == "date32":
            y, m, d = civil_from_days(c[n])
            _put_uint(buf, off, y, np.full(rows, 4, dtype=np.int64))
            buf[off + 4] = ord("-")
            _put_uint(buf, off + 5, m, np.full(rows, 2, dtype=np.int64))
            buf[off + 7] = ord("-")
            _put_uint(buf, off + 8, d, np.full(rows, 2, dtype=np.int64))
        else:
            lens_s, chars = c[n]
            pos = np.repeat(off, lens_s) + (np.arange(int(lens_s.sum()), dtype=np.int64)
                                            - np.repeat(np.cumsum(lens_s) - lens_s, lens_s))
            buf[pos] = chars
        buf[off + ln] = ord("|") if f + 1 < len(names) else ord("\n")
        off = off + ln + 1
    return buf.tobytes()


# The scan of the CSV workload: three range predicates (one date32, one
# decimal, one int32) with a joint selectivity of about 2%, fused with
# sum(d2 * i2) (int64 cents) and count(*).
CSV_T1_RANGE = (9131, 9769)       # 1995-01-01 .. 1996-09-30, ~25% of the dates
CSV_D1_LT = 2_000_000             # d1 < 20000.00: ~20%
CSV_I1_LT = 419_431               # i1 < 0.4 * 2^20: ~40%


def csv_scan_predicate():
    return and_(gte(col("t1"), num_lit(CSV_T1_RANGE[0], "date32")), lte(col("t1"), num_lit(CSV_T1_RANGE[1], "date32")),
                lt(col("d1"), num_lit(CSV_D1_LT, "int64")), lt(col("i1"), num_lit(CSV_I1_LT, "int32")))


# ----------------------------------------------------- high-cardinality group
#
# The serving form's group-by template: int64 keys drawn from n_keys distinct
# values with Zipf(s) frequencies (rank r has weight 1/r^s), one int64 value
# column. Ranks map to scattered int64 keys through an odd multiplier.

def zipf_keys(rows: int, n_keys: int, s: float = 1.1, seed: int = 5000) -> np.ndarray:
    ranks = np.arange(1, n_keys + 1, dtype=np.float64)
    cdf = np.cumsum(ranks ** -s)
    cdf /= cdf[-1]
    u = (splitmix64(seed * 1_000_003 + 1, rows) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    r = np.minimum(np.searchsorted(cdf, u, side="right"), n_keys - 1).astype(np.uint64)
    with np.errstate(over="ignore"):
        return ((r + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15) >> np.uint64(1)).astype(np.int64)


def groupby_table(rows: int, n_keys: int, s: float = 1.1, seed: int = 5000) -> Table:
    return Table([Column("k", "int64", zipf_keys(rows, n_keys, s, seed)),
                  Column("v", "int64", uniform(seed, 2, rows, -1_000_000, 1_000_000))])


def groupby_plan(groups_hint: int = 0) -> Plan:
    p = Plan()
    p.scan("scan", "t", ["k", "v"])
    p.group("group", "scan", ["k"], [aggregate("SUM", "s", col("v")), aggregate("COUNT", "c")],
            groups_hint=groups_hint)
    p.collate("collate", "group")
    return p


def csv_scan_plan(columns=("t1", "d1", "i1", "d2", "i2")) -> Plan:
    """Parse the lineitem text (input "lineitem"), apply the three range
    predicates and sum(d2 * i2), count(*)."""
    p = Plan()
    p.csv_scan("scan", "lineitem", LINEITEM_FIELDS, columns=list(columns), delimiter="|")
    p.filter("filter", "scan", csv_scan_predicate(), ["d2", "i2"])
    p.aggregate("agg", "filter", [aggregate("SUM", "sum_d2_i2", times(col("d2"), col("i2"))),
                                  aggregate("COUNT", "cnt")])
    p.collate("collate", "agg")
    return p
