"""The C ABI without a GPU: the library loads, exports every declared symbol,
and host-only entry points (plan validation, expression and spec compilation)
report errors the way the reference does (a status plus a message)."""

import ctypes
import re
from pathlib import Path

import pytest

from flexpushdowndb_gb300 import _abi, ops, plan, workloads
from flexpushdowndb_gb300.expression import and_, col, eq, gt, in_, lt, not_, num_lit, or_, str_lit, times
from flexpushdowndb_gb300.tupleset import Column, Table, export_host

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"\b(gfpdb_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    L = _abi.lib()
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(L, s), f"{s} declared in include/ but not exported"
        assert s in _abi.SIGNATURES, f"{s} has no ctypes signature"


def test_version_and_error_string():
    L = _abi.lib()
    assert L.gfpdb_version() >= 100
    assert isinstance(L.gfpdb_last_error(), bytes)


def test_plan_validation_accepts_workload_plans():
    plan.validate(workloads.two_table_plan())
    plan.validate(workloads.star_plan())


@pytest.mark.parametrize(
    "bad,fragment",
    [
        ('{"ops": []}', "CollatePOp"),
        ('{"ops": [{"type": "CollatePOp", "name": "c"}, {"type": "CollatePOp", "name": "c"}]}', "duplicate"),
        ('{"ops": [{"type": "FilterPOp", "name": "f", "predicate": {"type": "Sqrt"}, "consumers": ["c"]},'
         ' {"type": "CollatePOp", "name": "c"}]}', "Sqrt"),
        ('{"ops": [{"type": "TableScanPOp", "name": "s", "table": "t", "consumers": ["nope"]},'
         ' {"type": "CollatePOp", "name": "c"}]}', "unknown"),
        ('{"ops": [{"type": "HashJoinArrowPOp", "name": "j", "buildKey": "a", "probeKey": "b", "joinType": "SIDEWAYS"},'
         ' {"type": "CollatePOp", "name": "c"}]}', "SIDEWAYS"),
        ('{"ops": [{"type": "HashJoinArrowPOp", "name": "j", "buildKeys": ["a", "b"], "probeKeys": ["c", "d"],'
         ' "joinType": "LEFT"}, {"type": "CollatePOp", "name": "c"}]}', "one key column"),
        ("{not json", "JSON"),
    ],
)
def test_plan_validation_errors(bad, fragment):
    with pytest.raises(_abi.GfpdbError) as ei:
        plan.validate(bad)
    assert fragment in ei.value.message


def small_table():
    return Table([Column("a", "int32", [1, 2, 3]), Column("b", "int64", [4, 5, 6]),
                  Column("s", "utf8", ["x", "y", "z"]), Column("f", "float64", [0.5, 1.5, 2.5])])


@pytest.mark.parametrize(
    "pred",
    [
        lt(col("a"), num_lit(2)),
        and_(gt(col("b"), num_lit(4, "int64")), not_(eq(col("s"), str_lit("y")))),
        or_(in_(col("a"), [1, 3]), lt(times(col("a"), col("b")), num_lit(10, "int64"))),
        gt(col("f"), num_lit(1.0, "float64")),
        {"type": "Like", "left": col("s"), "right": str_lit("x%")},
        eq({"type": "Substr", "expr": col("s"), "fromLit": num_lit(1, "int64"), "forLit": num_lit(2, "int64")},
           str_lit("xy")),
        gt({"type": "DateExtract", "dateExpr": col("a"), "intervalType": "Year"}, num_lit(1970, "int64")),
        lt({"type": "If", "ifExpr": eq(col("s"), str_lit("x")), "thenExpr": col("a"), "elseExpr": col("b")},
           num_lit(3, "int64")),
    ],
)
def test_filter_compiles_without_gpu(pred):
    ops.Filter(pred, small_table())  # compile touches no device


@pytest.mark.parametrize(
    "pred,fragment",
    [
        (lt(col("missing"), num_lit(2)), "missing"),
        ({"type": "Like", "left": col("s"), "right": col("s")}, "pattern"),
        ({"type": "Like", "left": col("a"), "right": str_lit("%x")}, "utf8"),
        (eq({"type": "Substr", "expr": col("s"), "fromLit": col("a"), "forLit": num_lit(2)}, str_lit("x")), "literal"),
        (lt(col("s"), str_lit("x")), "strings"),
        (times(col("a"), col("b")), "boolean"),
    ],
)
def test_filter_compile_errors(pred, fragment):
    with pytest.raises(_abi.GfpdbError) as ei:
        ops.Filter(pred, small_table())
    assert fragment in ei.value.message


def test_group_spec_errors():
    with pytest.raises(_abi.GfpdbError):
        ops.Group(["a"], [{"function": "MEDIAN", "name": "m", "expr": col("a")}])
    with pytest.raises(_abi.GfpdbError):
        ops.Group(["a"], [{"function": "SUM", "name": "s"}])
    ops.Group(["a"], [ops.aggregate("SUM", "s", col("b")), ops.aggregate("COUNT", "c")])


def test_hashjoin_create_checks_types_and_keys():
    L = _abi.lib()
    h = ctypes.c_void_p()
    for jt in range(6):  # INNER .. RIGHT_SEMI
        assert L.gfpdb_hashjoin_create(jt, _abi.cstr_array(["a"]), _abi.cstr_array(["b"]), 1, None, -1, 0.5,
                                       ctypes.byref(h)) == 0
        L.gfpdb_hashjoin_free(h)
    rc = L.gfpdb_hashjoin_create(6, _abi.cstr_array(["a"]), _abi.cstr_array(["b"]), 1, None, -1, 0.5, ctypes.byref(h))
    assert rc == _abi.GFPDB_EINVAL
    two = _abi.cstr_array(["a", "b"])
    rc = L.gfpdb_hashjoin_create(1, two, two, 2, None, -1, 0.5, ctypes.byref(h))  # outer joins: one key column
    assert rc == _abi.GFPDB_EUNSUPPORTED
    for n in (0, 9):  # a key has 1 to 8 columns
        keys = _abi.cstr_array(["a"] * max(n, 1))
        rc = L.gfpdb_hashjoin_create(0, keys, keys, n, None, -1, 0.5, ctypes.byref(h))
        assert rc == _abi.GFPDB_EINVAL


def test_export_host_roundtrip_structure():
    t = small_table()
    ex = export_host(t)
    assert ex.schema.n_children == 4
    assert ex.array.array.length == 3
    assert ex.schema.children[2].contents.format == b"u"


def test_result_layout_of_an_exported_table():
    """gfpdb_result_layout reads any exported TupleSet's structure (host
    memory here): rows, names and formats, buffer pointers."""
    t = small_table()
    ex = export_host(t)
    L = _abi.lib()
    n, nc, dev = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
    names = ctypes.create_string_buffer(4096)
    vals, offs = (ctypes.c_void_p * 8)(), (ctypes.c_void_p * 8)()
    _abi.check(L.gfpdb_result_layout(ex.schema_ptr, ex.array_ptr, 8, ctypes.byref(n), ctypes.byref(nc),
                                     ctypes.byref(dev), names, 4096, vals, offs))
    assert (n.value, nc.value, dev.value) == (3, 4, _abi.ARROW_DEVICE_CPU)
    parts = names.raw.split(b"\0")[: 2 * nc.value]
    assert parts[0::2] == [c.name.encode() for c in t.columns]
    assert parts[1::2] == [ex.schema.children[i].contents.format for i in range(4)]
    for i in range(4):
        ca = ex.array.array.children[i].contents
        if parts[2 * i + 1] == b"u":
            assert (vals[i], offs[i]) == (ca.buffers[2], ca.buffers[1])
        else:
            assert vals[i] == ca.buffers[1] and offs[i] is None
    # too few columns allowed, or too little room for the names
    assert L.gfpdb_result_layout(ex.schema_ptr, ex.array_ptr, 3, ctypes.byref(n), ctypes.byref(nc),
                                 ctypes.byref(dev), names, 4096, vals, offs) == _abi.GFPDB_EINVAL
    assert L.gfpdb_result_layout(ex.schema_ptr, ex.array_ptr, 8, ctypes.byref(n), ctypes.byref(nc),
                                 ctypes.byref(dev), names, 4, vals, offs) == _abi.GFPDB_EINVAL


def test_prepared_launch_and_wait_argument_errors():
    """The prepared plan's launch / wait halves check their arguments before
    touching a device: null handles and outputs are EINVAL."""
    L = _abi.lib()
    n, gen = ctypes.c_int64(), ctypes.c_int64()
    assert L.gfpdb_prepared_launch(None, None) == _abi.GFPDB_EINVAL
    assert L.gfpdb_prepared_wait(None, None, ctypes.byref(n), ctypes.byref(gen)) == _abi.GFPDB_EINVAL
    assert L.gfpdb_prepared_run(None, None, None, ctypes.byref(n), ctypes.byref(gen)) == _abi.GFPDB_EINVAL
    assert b"null" in L.gfpdb_last_error()


def test_plan_validation_project_and_limit_sort():
    from flexpushdowndb_gb300.expression import col, divide

    p = plan.Plan()
    p.scan("scan", "t")
    p.project("proj", "scan", [("x", divide(col("a"), col("b")))], [("a", "a2")])
    p.limit_sort("top", "proj", 10, [("x", "DESC"), ("a2", "ASC")])
    p.collate("collate", "top")
    plan.validate(p)
    for k, order in ((1025, "ASC"), (-1, "ASC"), (10, "SIDEWAYS")):
        q = plan.Plan()
        q.scan("scan", "t")
        q.limit_sort("top", "scan", k, [("a", order)])
        q.collate("collate", "top")
        with pytest.raises(Exception):
            plan.validate(q)


def test_oracle_typed_joins():
    from oracle import ops as oops

    b = Table([Column("k", "int32", [1, 2, 2, 5]), Column("bv", "utf8", ["a", "b", "c", "d"])])
    p = Table([Column("fk", "int32", [2, 3, 1, 2]), Column("pv", "int64", [10, 20, 30, 40])])
    inner = [(1, 30, 1, "a"), (2, 10, 2, "b"), (2, 10, 2, "c"), (2, 40, 2, "b"), (2, 40, 2, "c")]
    assert oops.hash_join_typed(b, p, "k", "fk", "INNER").sorted_rows() == inner
    assert oops.hash_join_typed(b, p, "k", "fk", "LEFT").sorted_rows() == inner + [(None, None, 5, "d")]
    assert oops.hash_join_typed(b, p, "k", "fk", "RIGHT").sorted_rows() == inner + [(3, 20, None, None)]
    assert oops.hash_join_typed(b, p, "k", "fk", "FULL").sorted_rows() == inner + [(3, 20, None, None),
                                                                                   (None, None, 5, "d")]
    assert oops.hash_join_typed(b, p, "k", "fk", "LEFT_SEMI").sorted_rows() == [(1, "a"), (2, "b"), (2, "c")]
    assert oops.hash_join_typed(b, p, "k", "fk", "RIGHT_SEMI").sorted_rows() == [(1, 30), (2, 10), (2, 40)]


def test_oracle_limit_sort_is_stable():
    from oracle import ops as oops

    t = Table([Column("a", "int32", [3, 1, 3, 2, 1]), Column("i", "int32", [0, 1, 2, 3, 4])])
    assert oops.limit_sort(t, 3, [("a", "DESC")]).rows() == [(3, 0), (3, 2), (2, 3)]
    assert oops.limit_sort(t, 2, [("a", "ASC")]).rows() == [(1, 1), (1, 4)]


def test_plan_validation_shuffle_and_two_phase():
    from flexpushdowndb_gb300.expression import col

    aggs = [ops.aggregate("SUM", "s", col("a")), ops.aggregate("AVG", "m", col("b")), ops.aggregate("COUNT", "c")]
    p = plan.Plan()
    scans = [p.scan(f"scan{i}", f"t{i}") for i in range(3)]
    reduces = p.group_two_phase("g", scans, ["k"], aggs, 4)
    p._add({"type": "CollatePOp", "name": "collate"})
    for r in reduces:
        p.connect(r, "collate")
    plan.validate(p)
    assert [a["function"] for a in plan.partial_aggregates(aggs)] == ["SUM", "SUM", "COUNT", "COUNT"]
    assert [a["function"] for a in plan.reduce_aggregates(aggs)] == ["SUM", "AVG_REDUCE", "SUM"]
    bad = [
        ('{"ops": [{"type": "TableScanPOp", "name": "s", "table": "t", "consumers": ["sh"]},'
         ' {"type": "ShufflePOp", "name": "sh", "shuffleColumnNames": ["k"]},'
         ' {"type": "CollatePOp", "name": "c"}]}', "consumers"),
        ('{"ops": [{"type": "ShufflePOp", "name": "sh", "shuffleColumnNames": [], "consumers": ["c"]},'
         ' {"type": "CollatePOp", "name": "c"}]}', "1 to 8"),
        ('{"ops": [{"type": "GroupPOp", "name": "g", "groupColumnNames": ["k"], "consumers": ["c"],'
         ' "aggregates": [{"function": "AVG_REDUCE", "name": "m", "expr": {"type": "Column", "columnName": "x"}}]},'
         ' {"type": "CollatePOp", "name": "c"}]}', "AVG_REDUCE"),
    ]
    for text, fragment in bad:
        with pytest.raises(_abi.GfpdbError) as ei:
            plan.validate(text)
        assert fragment in ei.value.message


def test_shuffle_argument_checks_without_gpu():
    """Slot counts and key counts are checked before any device work."""
    L = _abi.lib()
    t = export_host(small_table())
    s, a = _abi.ArrowSchema(), _abi.ArrowDeviceArray()
    offs = (ctypes.c_int64 * 8)()
    for keys, slots in ((["a"], 0), (["a"], 1025), ([], 4)):
        rc = L.gfpdb_shuffle(t.schema_ptr, t.array_ptr, _abi.cstr_array(keys or ["a"]), len(keys), slots,
                             ctypes.byref(s), ctypes.byref(a), offs, None)
        assert rc == _abi.GFPDB_EINVAL


def test_oracle_shuffle_is_stable_and_complete():
    from oracle import ops as oops

    t = Table([Column("k", "int32", [5, 1, 5, 2, 1, 5, 9]), Column("i", "int32", list(range(7)))])
    rows, offs = oops.shuffle(t, ["k"], 3)
    assert offs[0] == 0 and offs[-1] == 7
    assert sorted(rows["i"].tolist()) == list(range(7))
    slots = oops.shuffle_slots(rows, ["k"], 3)
    assert list(slots) == sorted(slots)
    for s in range(3):
        ids = rows["i"][offs[s]:offs[s + 1]].tolist()
        assert ids == sorted(ids)


def test_malformed_arrow_schemas_are_refused():
    """A caller's ArrowSchema that breaks the C data interface's rules (no
    children array behind a positive count, a missing or released child, a
    negative count, a child without a format) is refused with
    GFPDB_EINVAL, never dereferenced."""
    import ctypes

    from flexpushdowndb_gb300.expression import col, lt, num_lit, to_json

    keep = []
    noop = _abi.SCHEMA_RELEASE(lambda p: None)
    keep.append(noop)

    def child(fmt, name, released=False):
        c = _abi.ArrowSchema()
        c.format = fmt
        c.name = name
        c.n_children = 0
        if not released:
            c.release = noop
        keep.append(c)
        return c

    def parent(children, n=None, null_array=False):
        s = _abi.ArrowSchema()
        s.format = b"+s"
        s.name = b""
        s.n_children = len(children) if n is None else n
        if not null_array:
            arr = (ctypes.POINTER(_abi.ArrowSchema) * max(1, len(children)))()
            for i, c in enumerate(children):
                arr[i] = ctypes.pointer(c) if c is not None else ctypes.POINTER(_abi.ArrowSchema)()
            s.children = ctypes.cast(arr, ctypes.POINTER(ctypes.POINTER(_abi.ArrowSchema)))
            keep.append(arr)
        s.release = noop
        keep.append(s)
        return s

    pred = to_json(lt(col("a"), num_lit(2))).encode()
    L = _abi.lib()
    h = ctypes.c_void_p()
    good = parent([child(b"i", b"a")])
    assert L.gfpdb_filter_compile(pred, ctypes.byref(good), ctypes.byref(h)) == 0
    L.gfpdb_filter_free(h)
    for bad in (parent([child(b"i", b"a")], null_array=True), parent([None]),
                parent([child(b"i", b"a", released=True)]), parent([child(b"i", b"a")], n=-1),
                parent([child(None, b"a")])):
        rc = L.gfpdb_filter_compile(pred, ctypes.byref(bad), ctypes.byref(h))
        assert rc == _abi.GFPDB_EINVAL, L.gfpdb_last_error()
