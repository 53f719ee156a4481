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


def test_layout_row_groups_match_pyarrow_metadata():
    """The host parser's row groups (offset of the first column chunk, rows)
    are those pyarrow recorded when it wrote each fixture."""
    from flexpushdowndb_gb300 import ops

    layout = json.loads((GOLDEN / "parquet" / "layout.json").read_text())
    for name, groups in layout.items():
        lay = ops.parquet_layout((GOLDEN / "parquet" / f"{name}.parquet").read_bytes())
        assert [{"offset": g["offset"], "rows": g["rows"]} for g in lay["rowGroups"]] == groups
        assert lay["numRows"] == sum(g["rows"] for g in groups)
        # a range read selects the row groups whose first chunk starts inside it
        if len(groups) > 1:
            part = ops.parquet_layout((GOLDEN / "parquet" / f"{name}.parquet").read_bytes(), ["i64"],
                                      groups[1]["offset"], groups[-1]["offset"])
            assert [g["offset"] for g in part["rowGroups"]] == [g["offset"] for g in groups[1:]]
            assert [c["name"] for c in part["columns"]] == ["i64"]


def _varint(v):
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        out.append(b | (0x80 if v else 0))
        if not v:
            return bytes(out)


def test_footer_with_a_huge_boolean_map_is_refused():
    """An unknown footer field holding a map of 2^40 boolean pairs: each
    pair is a byte of input, so the count runs into the footer's end at once
    (it must not be walked pair by pair without reading)."""
    from flexpushdowndb_gb300 import GfpdbError, ops

    footer = bytes([0x0B]) + _varint(20 << 1) + _varint(1 << 40) + bytes([0x11, 0x01, 0x01, 0x00])
    data = b"PAR1" + footer + len(footer).to_bytes(4, "little") + b"PAR1"
    with pytest.raises(GfpdbError):
        ops.parquet_layout(data)


def test_mutated_files_parse_or_are_refused():
    """Random byte changes in the fixtures' footers, anywhere in the file,
    in the footer length, and truncations: the host parser reads the file
    or refuses it with an error, never reading outside the buffer."""
    import random

    from flexpushdowndb_gb300 import GfpdbError, ops

    files = sorted((GOLDEN / "parquet").glob("*.parquet"))
    rng = random.Random(2024)
    outcomes = {"read": 0, "refused": 0}
    for _ in range(1500):
        b = bytearray(rng.choice(files).read_bytes())
        n = len(b)
        flen = int.from_bytes(b[n - 8:n - 4], "little")
        mode = rng.random()
        for _ in range(rng.randint(1, 8)):
            if mode < 0.6:
                i = rng.randrange(max(4, n - 8 - flen), n - 8)
            elif mode < 0.8:
                i = rng.randrange(n)
            else:
                i = rng.randrange(n - 8, n - 4)
            b[i] = rng.randrange(256)
        if rng.random() < 0.1:
            b = b[:rng.randrange(n)]
        try:
            ops.parquet_layout(bytes(b))
            outcomes["read"] += 1
        except GfpdbError:
            outcomes["refused"] += 1
    assert outcomes["read"] > 0 and outcomes["refused"] > 0
