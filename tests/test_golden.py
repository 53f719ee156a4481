"""Golden fixtures written by tests/golden/make_golden.py from pyarrow's own
hash join, hash aggregate, filter and CSV reader (an implementation
independent of both the oracle and the GPU path). The oracle must reproduce
every fixture (CPU); the GPU path must too (-m gpu)."""

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from flexpushdowndb_gb300 import workloads
from flexpushdowndb_gb300.expression import col
from flexpushdowndb_gb300.ops import aggregate
from oracle import ops as oops
from oracle import queries

GOLDEN = Path(__file__).resolve().parent / "golden"


def fixture(name):
    return json.loads((GOLDEN / f"{name}.json").read_text())


def rows(x):
    return sorted(tuple(r) for r in x)


def digest(rs):
    h = hashlib.sha256()
    for r in rs:
        h.update((",".join(str(v) for v in r) + "\n").encode())
    return h.hexdigest()


def star_inputs(f):
    if "parts" in f:
        tabs = workloads.batch_tables(len(f["parts"]), sizes=f["parts"], seed=f["seed"])
        return tabs, [f"p{i}" for i in range(len(f["parts"]))]
    return workloads.star_tables(fact_rows=f["fact_rows"], seed=f["seed"]), None


def groupby_check(f, got_rows):
    r = rows(got_rows)
    assert len(r) == f["groups"]
    assert sum(x[0] for x in r) == f["sum_keys"]
    assert sum(x[1] for x in r) == f["sum_sums"]
    assert sum(x[2] for x in r) == f["sum_counts"]
    assert digest(r) == f["digest"]


def csv_check(f, table):
    for n, v in f["column_sums"].items():
        assert int(np.asarray(table[n], dtype=np.int64).sum()) == v, n
    for n, d in f["string_digests"].items():
        assert digest([(s,) for s in table.column(n).to_list()]) == d, n


# ------------------------------------------------------------------ oracle


def test_oracle_two_table_golden():
    f = fixture("two_table_50k")
    t = workloads.two_table_tables(fact_rows=f["fact_rows"], seed=f["seed"])
    assert queries.two_table_query(t).sorted_rows() == rows(f["rows"])


@pytest.mark.parametrize("name", ["star_120k", "star_120k_consts_2_11_3_1", "star_ranges_3parts"])
def test_oracle_star_golden(name):
    f = fixture(name)
    tabs, parts = star_inputs(f)
    if parts is None:
        got = queries.star_query(tabs, consts=tuple(f["consts"]))
    else:
        got = queries.star_query_ranges(tabs, parts, [tuple(r) for r in f["ranges"]])
    assert got.sorted_rows() == rows(f["rows"])


def test_oracle_csv_golden():
    f = fixture("csv_scan_20k")
    text = workloads.lineitem_csv(f["rows"], f["seed"])
    assert len(text) == f["text_bytes"]
    t = oops.csv_parse(text, workloads.LINEITEM_FIELDS, delimiter="|")
    csv_check(f, t)
    sel = oops.filter_table(t, workloads.csv_scan_predicate())
    assert sel.num_rows == f["selected"]
    assert int((np.asarray(sel["d2"], dtype=np.int64) * np.asarray(sel["i2"], dtype=np.int64)).sum()) == f["sum_d2_i2"]


def test_oracle_groupby_golden():
    f = fixture("groupby_300k")
    t = workloads.groupby_table(f["rows"], f["n_keys"], seed=f["seed"])
    g = oops.group_by(t, ["k"], [{"function": "SUM", "name": "s", "expr": col("v")},
                                 {"function": "COUNT", "name": "c"}])
    groupby_check(f, g.rows())


# --------------------------------------------------------------------- GPU


@pytest.mark.gpu
def test_gpu_two_table_golden(gpu):
    from flexpushdowndb_gb300 import plan

    f = fixture("two_table_50k")
    t = workloads.two_table_tables(fact_rows=f["fact_rows"], seed=f["seed"])
    assert plan.execute(workloads.two_table_plan(), t).table.sorted_rows() == rows(f["rows"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["star_120k", "star_120k_consts_2_11_3_1", "star_ranges_3parts"])
def test_gpu_star_golden(gpu, name):
    from flexpushdowndb_gb300 import batch, plan
    from flexpushdowndb_gb300.tupleset import DeviceTable

    f = fixture(name)
    tabs, parts = star_inputs(f)
    if parts is None:
        got = plan.execute(workloads.star_plan(consts=tuple(f["consts"])), tabs).table.sorted_rows()
        assert got == rows(f["rows"])
    else:
        ranges = [tuple(r) for r in f["ranges"]]
        got = plan.execute(workloads.star_plan(ranges=ranges, fact_tables=parts), tabs).table.sorted_rows()
        assert got == rows(f["rows"])
        dev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
        b = batch.split_by_query(batch.star_batch(workloads.star_batch_spec(parts, [ranges]), dev).table)
        assert b.get(0, []) == rows(f["rows"])


@pytest.mark.gpu
def test_gpu_csv_golden(gpu):
    from flexpushdowndb_gb300 import ops

    f = fixture("csv_scan_20k")
    text = workloads.lineitem_csv(f["rows"], f["seed"])
    t = ops.csv_read(text, workloads.LINEITEM_FIELDS, delimiter="|")
    csv_check(f, t)
    fl = ops.Filter(workloads.csv_scan_predicate(), t)
    sel = ops.select(t, fl, project=["d2", "i2"])
    assert sel.num_rows == f["selected"]
    assert int((np.asarray(sel["d2"], dtype=np.int64) * np.asarray(sel["i2"], dtype=np.int64)).sum()) == f["sum_d2_i2"]


@pytest.mark.gpu
def test_gpu_groupby_golden(gpu):
    from flexpushdowndb_gb300 import plan

    f = fixture("groupby_300k")
    t = workloads.groupby_table(f["rows"], f["n_keys"], seed=f["seed"])
    got = plan.execute(workloads.groupby_plan(), {"t": t}).table
    groupby_check(f, got.rows())


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
def test_gpu_csv_scan_plan_golden(gpu, graph):
    """CsvScanPOp -> FilterPOp -> AggregatePOp as one plan."""
    from flexpushdowndb_gb300 import plan
    from flexpushdowndb_gb300.tupleset import text_table

    f = fixture("csv_scan_20k")
    text = workloads.lineitem_csv(f["rows"], f["seed"])
    p = json.loads(workloads.csv_scan_plan().to_json())
    p["cudaGraph"] = graph
    for _ in range(2):
        got = plan.execute(json.dumps(p), {"lineitem": text_table(text)}).table
        assert got.names == ["sum_d2_i2", "cnt"]
        assert got.rows() == [(f["sum_d2_i2"], f["selected"])]


def test_c_baselines_golden():
    """The timed CPU baselines (oracle/baseline.c) reproduce the fixtures."""
    from oracle import cbaseline

    f = fixture("csv_scan_20k")
    text = workloads.lineitem_csv(f["rows"], f["seed"])
    s, n = cbaseline.csv_scan(text, workloads.CSV_T1_RANGE, workloads.CSV_D1_LT, workloads.CSV_I1_LT, threads=3)
    assert (s, n) == (f["sum_d2_i2"], f["selected"])
    f = fixture("star_120k")
    tabs = workloads.star_tables(fact_rows=f["fact_rows"], seed=f["seed"])
    got = cbaseline.star_query(cbaseline.StarInputs(tabs), consts=tuple(f["consts"]), threads=3)
    assert got.sorted_rows() == rows(f["rows"])


def test_c_baseline_full_size_golden():
    """The C port (the reference arm of the benchmark) at full size: the star
    query over 6,000,000 fact rows, and all 32 variants of the batched form
    over its 64 partitions (59,952,713 rows)."""
    from oracle import cbaseline

    f = fixture("star_6m")
    tabs = workloads.star_tables(fact_rows=f["fact_rows"], seed=f["seed"])
    got = cbaseline.star_query(cbaseline.StarInputs(tabs), consts=tuple(f["consts"]))
    assert got.sorted_rows() == rows(f["rows"])
    del tabs
    f = fixture("star_batch_64x32")
    tabs = workloads.batch_tables(f["parts"])
    inp = cbaseline.StarInputs(tabs, parts=[f"p{i}" for i in range(f["parts"])])
    assert inp.rows == f["fact_rows"]
    for v in f["variants"]:
        got = cbaseline.star_query_ranges(inp, v["ranges"]).sorted_rows()
        assert len(got) == v["groups"] and digest(got) == v["digest"]
