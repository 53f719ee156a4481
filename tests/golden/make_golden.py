"""Writes the golden fixtures in this directory from pyarrow (25.x): Arrow's
own hash join, hash aggregate, compute filter and CSV reader on the seeded
synthetic workloads, an implementation independent of both the oracle and
the GPU path. Run here (pyarrow is a dependency of this script only; the
fixtures are what the tests read):

    python tests/golden/make_golden.py           # small fixtures
    python tests/golden/make_golden.py --full    # the workloads at full size

Each fixture records the workload parameters (the inputs are regenerated
from the seeds by flexpushdowndb_gb300.workloads) and the expected result:
all rows for small results, else size-independent checksums.
"""

from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pyarrow as pa
import pyarrow.compute as pc
import pyarrow.csv as pcsv

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from flexpushdowndb_gb300 import workloads  # noqa: E402


def arrow(t) -> pa.Table:
    cols = {}
    for c in t.columns:
        if c.type == "utf8":
            cols[c.name] = pa.array(list(c.values) if not isinstance(c.values, tuple) else c.to_list(), pa.string())
        else:
            cols[c.name] = pa.array(np.asarray(c.values, dtype=np.int64), pa.int64())
    return pa.table(cols)


def rows_of(t: pa.Table, names) -> list:
    cols = [t.column(n).to_pylist() for n in names]
    return sorted(tuple(r) for r in zip(*cols))


def digest(rows) -> str:
    h = hashlib.sha256()
    for r in rows:
        h.update((",".join(str(x) for x in r) + "\n").encode())
    return h.hexdigest()


def two_table(fact_rows=50_000, seed=1000):
    t = workloads.two_table_tables(fact_rows=fact_rows, seed=seed)
    dim = arrow(t["dim"]).filter(pc.less(pc.field("category"), 5)).select(["pk", "region"])
    fact = arrow(t["fact"])
    j = fact.join(dim, keys="fk", right_keys="pk", join_type="inner")
    j = j.append_column("rev", pc.multiply(j["price_cents"], j["qty"]))
    g = j.group_by("region").aggregate([("rev", "sum"), ("rev", "count")])
    return {"query": "two_table", "fact_rows": fact_rows, "seed": seed,
            "columns": ["region", "revenue", "cnt"],
            "rows": rows_of(g.rename_columns(["region", "revenue", "cnt"]), ["region", "revenue", "cnt"])}


def star(fact_rows=120_000, seed=2000, consts=(1, 3, 2, 5), ranges=None, parts=None):
    if parts is None:
        tabs = workloads.star_tables(fact_rows=fact_rows, seed=seed)
        cur = arrow(tabs["fact"])
    else:
        tabs = workloads.batch_tables(len(parts), sizes=parts, seed=seed)
        cur = pa.concat_tables([arrow(tabs[f"p{i}"]) for i in range(len(parts))])
    for i in range(1, 5):
        d = arrow(tabs[f"d{i}"])
        f = d[f"d{i}_f"]
        if ranges is None:
            mask = pc.equal(f, consts[i - 1])
        else:
            lo, hi = ranges[i - 1]
            mask = pc.and_(pc.greater_equal(f, lo), pc.less_equal(f, hi))
        keep = [f"d{i}_pk", f"d{i}_g"] if i in (2, 4) else [f"d{i}_pk"]
        d = d.filter(mask).select(keep)
        cur = cur.join(d, keys=f"fk{i}", right_keys=f"d{i}_pk", join_type="inner")
    cur = cur.append_column("rev", pc.multiply(cur["price_cents"], cur["qty"]))
    cur = cur.append_column("drev", pc.multiply(cur["price_cents"], cur["discount"]))
    g = cur.group_by(["d2_g", "d4_g"]).aggregate([("rev", "sum"), ("drev", "sum"), ("rev", "count")])
    names = ["d2_g", "d4_g", "revenue", "discount_revenue", "cnt"]
    g = g.select(["d2_g", "d4_g", "rev_sum", "drev_sum", "rev_count"]).rename_columns(names)
    out = {"query": "star", "seed": seed, "columns": names, "rows": rows_of(g, names)}
    if parts is None:
        out.update(fact_rows=fact_rows, consts=list(consts))
    else:
        out.update(parts=list(parts), ranges=[list(r) for r in ranges])
    return out


def decimal_cents(col) -> np.ndarray:
    """Unscaled values of a decimal128 column (its two's-complement 128-bit
    storage; every value here fits the low 64 bits)."""
    a = col.combine_chunks() if hasattr(col, "combine_chunks") else col
    words = np.frombuffer(a.buffers()[1], dtype=np.int64)
    return words[2 * a.offset: 2 * (a.offset + len(a)): 2].copy()


def csv_scan(rows=20_000, seed=workloads.CSV_SEED):
    text = workloads.lineitem_csv(rows, seed)
    names = [n for n, _ in workloads.LINEITEM_FIELDS]
    types = {}
    for n, ty in workloads.LINEITEM_FIELDS:
        types[n] = (pa.int32() if ty == "int32" else pa.decimal128(15, 2) if ty.startswith("decimal")
                    else pa.date32() if ty == "date32" else pa.string())
    t = pcsv.read_csv(pa.BufferReader(text), read_options=pcsv.ReadOptions(column_names=names),
                      parse_options=pcsv.ParseOptions(delimiter="|"),
                      convert_options=pcsv.ConvertOptions(column_types=types))
    cents = {n: decimal_cents(t[n]) for n, ty in workloads.LINEITEM_FIELDS if ty.startswith("decimal")}
    days = {n: t[n].cast(pa.int32()).to_numpy().astype(np.int64) for n in ("t1", "t2")}
    ints = {n: t[n].to_numpy().astype(np.int64) for n in ("i1", "i2", "i3", "i4")}
    col_sums = {n: int(v.sum()) for n, v in {**ints, **cents, **days}.items()}
    str_digest = {n: digest([(s,) for s in t[n].to_pylist()]) for n in ("s1", "s2", "s3", "s4", "s5", "s6")}
    lo, hi = workloads.CSV_T1_RANGE
    m = (days["t1"] >= lo) & (days["t1"] <= hi) & (cents["d1"] < workloads.CSV_D1_LT) & (ints["i1"] < workloads.CSV_I1_LT)
    return {"query": "csv_scan", "rows": rows, "seed": seed, "text_bytes": len(text), "column_sums": col_sums,
            "string_digests": str_digest, "selected": int(m.sum()),
            "sum_d2_i2": int((cents["d2"][m] * ints["i2"][m]).sum())}


def groupby(rows=300_000, n_keys=1_000_000, seed=5000):
    t = arrow(workloads.groupby_table(rows, n_keys, seed=seed))
    g = t.group_by("k").aggregate([("v", "sum"), ("v", "count")])
    r = rows_of(g.rename_columns(["k", "s", "c"]), ["k", "s", "c"])
    return {"query": "groupby", "rows": rows, "n_keys": n_keys, "seed": seed, "groups": len(r),
            "sum_keys": int(sum(x[0] for x in r)), "sum_sums": int(sum(x[1] for x in r)),
            "sum_counts": int(sum(x[2] for x in r)), "digest": digest(r)}


def star_batch(n_parts=64, n_queries=32):
    """The batched form at full size: every query variant of
    workloads.batch_queries over the 64-partition fact table, each run as its
    own chain of Arrow joins and one hash aggregate; per variant its group
    count, row digest and column sums."""
    tabs = workloads.batch_tables(n_parts)
    fact = pa.concat_tables([arrow(tabs[f"p{i}"]) for i in range(n_parts)])
    dims = {i: arrow(tabs[f"d{i}"]) for i in range(1, 5)}
    out = []
    for q in workloads.batch_queries(n_queries):
        cur = fact
        for i in range(1, 5):
            lo, hi = q[i - 1]
            d = dims[i]
            f = d[f"d{i}_f"]
            keep = [f"d{i}_pk", f"d{i}_g"] if i in (2, 4) else [f"d{i}_pk"]
            d = d.filter(pc.and_(pc.greater_equal(f, lo), pc.less_equal(f, hi))).select(keep)
            cur = cur.join(d, keys=f"fk{i}", right_keys=f"d{i}_pk", join_type="inner")
        cur = cur.append_column("rev", pc.multiply(cur["price_cents"], cur["qty"]))
        cur = cur.append_column("drev", pc.multiply(cur["price_cents"], cur["discount"]))
        g = cur.group_by(["d2_g", "d4_g"]).aggregate([("rev", "sum"), ("drev", "sum"), ("rev", "count")])
        names = ["d2_g", "d4_g", "revenue", "discount_revenue", "cnt"]
        r = rows_of(g.select(["d2_g", "d4_g", "rev_sum", "drev_sum", "rev_count"]).rename_columns(names), names)
        out.append({"ranges": [list(x) for x in q], "groups": len(r), "digest": digest(r),
                    "sum_revenue": int(sum(x[2] for x in r)), "sum_discount_revenue": int(sum(x[3] for x in r)),
                    "sum_cnt": int(sum(x[4] for x in r))})
        print("variant", len(out), len(r), flush=True)
    return {"query": "star_batch", "parts": n_parts, "seed": workloads.BATCH_SEED,
            "fact_rows": fact.num_rows, "columns": ["d2_g", "d4_g", "revenue", "discount_revenue", "cnt"],
            "variants": out}


def full_size():
    """Fixtures of the workloads at their full sizes (size-independent
    checksums where the result is large)."""
    return {
        "two_table_1m": two_table(fact_rows=1_000_000),
        "star_6m": star(fact_rows=6_000_000),
        "csv_scan_6m": csv_scan(rows=6_000_000),
        "star_batch_64x32": star_batch(),
    }


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--full":
        fixtures = full_size()
        for name, f in fixtures.items():
            (HERE / f"{name}.json").write_text(json.dumps(f, separators=(",", ":")) + "\n")
            print(name, len(json.dumps(f)))
        return
    fixtures = {
        "two_table_50k": two_table(),
        "star_120k": star(),
        "star_120k_consts_2_11_3_1": star(consts=(2, 11, 3, 1), seed=2013),
        "star_ranges_3parts": star(seed=4070, parts=[5_000, 70_001, 2_049],
                                   ranges=[(0, 39), (0, 24), (3, 50), (0, 99)]),
        "csv_scan_20k": csv_scan(),
        "groupby_300k": groupby(),
    }
    for name, f in fixtures.items():
        (HERE / f"{name}.json").write_text(json.dumps(f, separators=(",", ":")) + "\n")
        print(name, len(json.dumps(f)))


if __name__ == "__main__":
    main()
