"""The Parquet fixtures hold the seeded tables they were written from
(checked with pyarrow where it is installed), and the plan operators that
read Parquet validate on the host."""

import json
import sys
from pathlib import Path

import pytest

from flexpushdowndb_gb300 import _abi, plan

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from parquet_source import FIXTURES, source  # noqa: E402


@pytest.mark.parametrize("name", list(FIXTURES))
def test_fixture_holds_its_source(name):
    pq = pytest.importorskip("pyarrow.parquet")
    n, seed, _, required = FIXTURES[name]
    t = pq.read_table(GOLDEN / "parquet" / f"{name}.parquet")
    assert t.num_rows == n
    for col, (ty, vals) in source(n, seed).items():
        got = t.column(col).to_pylist()
        if ty == "date32":
            got = [(d - __import__("datetime").date(1970, 1, 1)).days for d in got]
        assert got == (list(vals) if ty == "utf8" else vals.tolist()), col
        assert t.schema.field(col).nullable == (not required)


def test_layout_lists_every_fixture():
    layout = json.loads((GOLDEN / "parquet" / "layout.json").read_text())
    assert set(layout) == set(FIXTURES)
    for name, groups in layout.items():
        assert sum(g["rows"] for g in groups) == FIXTURES[name][0]


def test_parquet_plan_operators_validate():
    p = plan.Plan()
    p._add({"type": "ParquetScanPOp", "name": "s", "table": "f", "columns": ["a"]})
    p._add({"type": "FileScanPOp", "name": "t", "path": "/nonexistent.parquet", "format": "parquet"})
    p.collate("c", "s")
    p.connect("t", "c")
    plan.validate(p)
    q = plan.Plan()
    q._add({"type": "FileScanPOp", "name": "t", "path": "x", "format": "orc"})
    q.collate("c", "t")
    with pytest.raises(_abi.GfpdbError):
        plan.validate(q)


def test_package_writer_is_read_by_pyarrow():
    import io

    import numpy as np

    pq = pytest.importorskip("pyarrow.parquet")
    from flexpushdowndb_gb300.parquet_writer import write_parquet
    from flexpushdowndb_gb300.tupleset import Column, Table

    n, seed, _, _ = FIXTURES["plain_none_v1"]
    cols = source(n, seed)
    t = Table([Column(k, ty, v) for k, (ty, v) in cols.items()])
    for kw in (dict(), dict(dictionary_max=0), dict(row_group_rows=3000, page_rows=700)):
        back = pq.read_table(io.BytesIO(write_parquet(t, **kw)))
        for c in t.columns:
            got = back.column(c.name).to_pylist()
            if c.type == "date32":
                got = [(d - __import__("datetime").date(1970, 1, 1)).days for d in got]
            if c.type == "float64":
                assert np.array_equal(np.array(got).view(np.int64), c.values.view(np.int64))
            else:
                assert got == c.to_list(), c.name
