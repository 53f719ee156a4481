"""The Parquet reader (gfpdb_parquet_read, ParquetScanPOp, FileScanPOp) on
the GPU path against the values the fixtures were written from
(tests/golden/parquet_source.py; tests/golden/make_parquet.py wrote them
with pyarrow): every column type, plain and dictionary pages, no compression
and snappy, data pages v1 and v2, several row groups and many pages,
optional and required columns, column selection, row-group ranges, and the
files the reader refuses."""

import json
import sys
from pathlib import Path

import numpy as np
import pytest

from flexpushdowndb_gb300 import GfpdbError, ops, plan
from flexpushdowndb_gb300.expression import col, gt, num_lit
from flexpushdowndb_gb300.tupleset import Column, Table, text_table
from oracle import ops as oops

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from parquet_source import FIXTURES, source  # noqa: E402

LAYOUT = json.loads((GOLDEN / "parquet" / "layout.json").read_text())


def expected(name, rows=None):
    n, seed, _, _ = FIXTURES[name]
    cols = source(n, seed)
    t = Table([Column(k, ty, v) for k, (ty, v) in cols.items()])
    if rows is not None:
        t = t.slice(*rows)
    return t


def same(got: Table, want: Table):
    assert got.names == want.names
    assert [c.type for c in got.columns] == [c.type for c in want.columns]
    for g, w in zip(got.columns, want.columns):
        if g.type == "float64":
            assert np.array_equal(g.values.view(np.int64), w.values.view(np.int64))  # bit for bit
        else:
            assert g.to_list() == w.to_list(), g.name


@pytest.mark.parametrize("name", list(FIXTURES))
def test_read_whole_file(gpu, name):
    path = GOLDEN / "parquet" / f"{name}.parquet"
    same(ops.parquet_read(path.read_bytes()), expected(name))
    same(ops.parquet_read(path), expected(name))  # from the file system


@pytest.mark.parametrize("name", ["dict_snappy_v1", "plain_snappy_v2", "required_dict_none"])
def test_column_selection_and_order(gpu, name):
    path = GOLDEN / "parquet" / f"{name}.parquet"
    got = ops.parquet_read(path.read_bytes(), ["u", "k", "d"])
    want = expected(name)
    same(got, Table([want.column("u"), want.column("k"), want.column("d")]))


@pytest.mark.parametrize("name", ["plain_none_v1", "dict_snappy_v1", "dict_snappy_v2"])
def test_row_group_ranges(gpu, name):
    """readRange: the row groups whose first column chunk starts in the range."""
    groups = LAYOUT[name]
    data = (GOLDEN / "parquet" / f"{name}.parquet").read_bytes()
    starts = np.cumsum([0] + [g["rows"] for g in groups])
    for i, g in enumerate(groups):
        got = ops.parquet_read(data, ["i64", "s"], g["offset"], g["offset"])
        want = expected(name, (int(starts[i]), int(starts[i + 1])))
        same(got, Table([want.column("i64"), want.column("s")]))
    last = groups[-1]["offset"]
    got = ops.parquet_read(data, ["i32"], groups[1]["offset"], last)
    same(got, Table([expected(name, (int(starts[1]), int(starts[-1]))).column("i32")]))


@pytest.mark.parametrize("name,cols,fragment", [
    ("nulls", None, "null"), ("gzip", None, "codec"), ("bools", None, "BOOLEAN"), ("plain_none_v1", ["zz"], "zz"),
])
def test_refused_files(gpu, name, cols, fragment):
    with pytest.raises(GfpdbError) as ei:
        ops.parquet_read((GOLDEN / "parquet" / f"{name}.parquet").read_bytes(), cols)
    assert fragment in ei.value.message


def test_readable_columns_beside_a_refused_one(gpu):
    got = ops.parquet_read((GOLDEN / "parquet" / "bools.parquet").read_bytes(), ["x"])
    assert got["x"].tolist() == list(range(500))


def test_not_parquet(gpu):
    with pytest.raises(GfpdbError):
        ops.parquet_read(b"PAR1 this is not parquet at all PAR1")


@pytest.mark.parametrize("via", ["table", "file"])
def test_parquet_scans_in_plans(gpu, via):
    name = "dict_snappy_v2"
    path = GOLDEN / "parquet" / f"{name}.parquet"
    p = plan.Plan()
    if via == "table":
        p._add({"type": "ParquetScanPOp", "name": "scan", "table": "file", "columns": ["k", "i64", "s"]})
        tables = {"file": text_table(path.read_bytes())}
    else:
        p._add({"type": "FileScanPOp", "name": "scan", "path": str(path), "format": "parquet",
                "columns": ["k", "i64", "s"]})
        tables = {}
    p.filter("f", "scan", gt(col("i64"), num_lit(0, "int64")))
    p.group("g", "f", ["k", "s"], [ops.aggregate("COUNT", "n"), ops.aggregate("MAX", "hi", col("i64"))])
    p.collate("collate", "g")
    got = plan.execute(p, tables).table
    want = oops.group_by(oops.filter_table(expected(name), gt(col("i64"), num_lit(0, "int64"))), ["k", "s"],
                         [ops.aggregate("COUNT", "n"), ops.aggregate("MAX", "hi", col("i64"))])
    assert got.sorted_rows() == want.sorted_rows()


def test_csv_file_scan(gpu, tmp_path):
    path = tmp_path / "t.csv"
    path.write_text("1,5,x\n2,6,yy\n3,7,zzz\n")
    p = plan.Plan()
    p._add({"type": "FileScanPOp", "name": "scan", "path": str(path), "format": "csv",
            "fields": [{"name": "a", "type": "int32"}, {"name": "b", "type": "int64"}, {"name": "c", "type": "utf8"}],
            "columns": ["c", "a"]})
    p.collate("collate", "scan")
    assert plan.execute(p, {}).table.rows() == [("x", 1), ("yy", 2), ("zzz", 3)]


@pytest.mark.parametrize("kw", [dict(), dict(dictionary_max=0), dict(row_group_rows=3000, page_rows=700)])
def test_reads_the_package_writer(gpu, kw):
    """Files of flexpushdowndb_gb300.parquet_writer (REQUIRED columns,
    plain or bit-packed dictionary pages) read back as written."""
    from flexpushdowndb_gb300.parquet_writer import write_parquet

    want = expected("plain_none_v1")
    got = ops.parquet_read(write_parquet(want, **kw))
    same(got, want)


@pytest.mark.parametrize("ty", ["int32", "int64", "utf8"])
def test_dictionary_index_out_of_range(gpu, ty, monkeypatch):
    """A data page whose dictionary index names no dictionary entry (every
    index one past the value written, so the largest is one past the
    dictionary; the bit width still holds it) is refused as malformed, for
    fixed-width columns (decoded to values in the page pass) and byte-array
    columns (looked up in the values pass) alike."""
    from flexpushdowndb_gb300 import parquet_writer as pw

    vals = np.arange(3000) % 3  # three distinct values: two-bit indices 0..2
    column = Column("c", ty, [f"s{v}" for v in vals] if ty == "utf8" else vals)
    t = Table([column])
    assert ops.parquet_read(pw.write_parquet(t)).column("c").to_list() == column.to_list()
    orig = pw._bitpacked
    monkeypatch.setattr(pw, "_bitpacked", lambda idx, bw: orig(idx + 1, bw))
    bad = pw.write_parquet(t)
    with pytest.raises(GfpdbError) as ei:
        ops.parquet_read(bad)
    assert "malformed" in ei.value.message
