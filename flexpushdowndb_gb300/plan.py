"""Physical plans of the reference's operators, run by gfpdb_execute_plan.

A plan is a JSON list of operators in the reference's vocabulary
(TableScanPOp, FilterPOp, BloomFilterCreatePOp, BloomFilterUsePOp,
HashJoinArrowPOp, GroupPOp, CollatePOp) with their consumers; the library
derives producers, runs the operators' message protocol on one GPU and
returns the CollatePOp's TupleSet.
"""

from __future__ import annotations

import ctypes
import json
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _abi
from .expression import Expr
from .tupleset import (NP_TYPES, TYPES, Column, DeviceTable, Exported, ResultReader, Table, export_host,
                       import_result, new_output)


class Plan:
    def __init__(self):
        self.ops: list[dict] = []

    def _add(self, op: dict) -> str:
        self.ops.append(op)
        return op["name"]

    def op(self, name: str) -> dict:
        for o in self.ops:
            if o["name"] == name:
                return o
        raise KeyError(name)

    def connect(self, producer: str, consumer: str) -> None:
        cons = self.op(producer).setdefault("consumers", [])
        if consumer not in cons:
            cons.append(consumer)

    def scan(self, name: str, table: str, columns: Sequence[str] | None = None, chunk_rows: int = 0,
             in_place: Sequence[str] = ()) -> str:
        """TableScanPOp. `in_place`: columns of a page-locked host table the
        kernels read over the chip-to-chip link instead of a copy."""
        op = {"type": "TableScanPOp", "name": name, "table": table}
        if columns:
            op["columns"] = list(columns)
        if chunk_rows:
            op["chunkRows"] = chunk_rows
        if in_place:
            op["inPlaceColumns"] = list(in_place)
        return self._add(op)

    def filter(self, name: str, producer: str, predicate: Expr, project: Sequence[str] | None = None) -> str:
        op = {"type": "FilterPOp", "name": name, "predicate": predicate}
        if project:
            op["projectColumnNames"] = list(project)
        self._add(op)
        self.connect(producer, name)
        return name

    def bloom_create(self, name: str, producer: str, column: str, bits_per_key: int = 10, num_hashes: int = 3) -> str:
        self._add({"type": "BloomFilterCreatePOp", "name": name, "bloomFilterColumn": column,
                   "bitsPerKey": bits_per_key, "numHashes": num_hashes, "bloomFilterUsePOps": []})
        self.connect(producer, name)
        return name

    def bloom_use(self, name: str, producer: str, creator: str, column: str) -> str:
        self._add({"type": "BloomFilterUsePOp", "name": name, "bloomFilterColumn": column})
        self.connect(producer, name)
        self.op(creator)["bloomFilterUsePOps"].append(name)
        return name

    def hash_join(self, name: str, build: str, probe: str, build_key: str | Sequence[str],
                  probe_key: str | Sequence[str], project: Sequence[str] | None = None, load_factor: float = 0.5,
                  join_type: str = "INNER") -> str:
        """HashJoinArrowPOp. Keys are one column per side, or equal-length
        lists (HashJoinPredicate's column lists); `join_type` is one of
        INNER, LEFT (every build row kept), RIGHT (every probe row kept),
        FULL, LEFT_SEMI (matched build rows), RIGHT_SEMI (matched probe
        rows)."""
        op = {"type": "HashJoinArrowPOp", "name": name, "buildProducers": [build], "probeProducers": [probe],
              "joinType": join_type, "loadFactor": load_factor}
        if isinstance(build_key, str) and isinstance(probe_key, str):
            op["buildKey"], op["probeKey"] = build_key, probe_key
        else:
            bk = [build_key] if isinstance(build_key, str) else list(build_key)
            pk = [probe_key] if isinstance(probe_key, str) else list(probe_key)
            if not bk or len(bk) != len(pk):
                raise ValueError("a hash join needs as many probe keys as build keys, at least one")
            op["buildKeys"], op["probeKeys"] = bk, pk
        if project:
            op["projectColumnNames"] = list(project)
        self._add(op)
        self.connect(build, name)
        self.connect(probe, name)
        return name

    def group(self, name: str, producer: str, group_columns: Sequence[str], aggregates: Sequence[dict],
              groups_hint: int = 0) -> str:
        self._add({"type": "GroupPOp", "name": name, "groupColumnNames": list(group_columns),
                   "aggregates": list(aggregates), "groupsHint": groups_hint})
        self.connect(producer, name)
        return name

    def aggregate(self, name: str, producer: str, aggregates: Sequence[dict]) -> str:
        """Non-grouped aggregate (AggregatePOp)."""
        self._add({"type": "AggregatePOp", "name": name, "aggregates": list(aggregates)})
        self.connect(producer, name)
        return name

    def shuffle(self, name: str, producer: str, columns: Sequence[str], consumers: Sequence[str] = ()) -> str:
        """ShufflePOp: rows hash-partitioned on `columns`, slot i to the i-th
        consumer (consumers may also be connected later, in slot order)."""
        self._add({"type": "ShufflePOp", "name": name, "shuffleColumnNames": list(columns)})
        self.connect(producer, name)
        for c in consumers:
            self.connect(name, c)
        return name

    def group_two_phase(self, name: str, producers: Sequence[str], group_columns: Sequence[str],
                        aggregates: Sequence[dict], parallel_degree: int) -> list[str]:
        """The parallel group-by of PrePToPTransformer::transformGroupTwoPhase
        (fpdb-executor/src/physical/transform/PrePToPTransformer.cpp:434-580):
        a partial GroupPOp per producer, a ShufflePOp on the group columns
        after each, and `parallel_degree` reduce GroupPOps fed by every
        shuffle. AVG becomes an intermediate SUM and COUNT, reduced by
        AVG_REDUCE; SUM and COUNT reduce by SUM, MIN and MAX by themselves
        (PrePToPTransformerUtil.cpp:63-124). Returns the reduce ops' names,
        each holding a disjoint set of groups."""
        partial, reduce = partial_aggregates(aggregates), reduce_aggregates(aggregates)
        reduces = [f"{name}-reduce-{i}" for i in range(parallel_degree)]
        shuffles = []
        for i, p in enumerate(producers):
            g = self.group(f"{name}-{i}", p, group_columns, partial)
            shuffles.append(self.shuffle(f"{name}-shuffle-{i}", g, group_columns))
        for r in reduces:
            self._add({"type": "GroupPOp", "name": r, "groupColumnNames": list(group_columns), "aggregates": reduce})
            for sh in shuffles:
                self.connect(sh, r)
        return reduces

    def predicate_transfer(self, tables: dict[str, int | tuple[int, float]], joins: Sequence[dict],
                           bits_per_key: int = 10, num_hashes: int = 3, prefix: str = "pt") -> dict[str, str]:
        """Add the bloom-filter predicate transfer of a join graph
        (gfpdb_plan_predicate_transfer, SmallToLargePredTransOrder):
        `tables` maps the operator producing each base table to its row
        count, or to (row count, selectivity of its local filters); `joins` are {"left", "right", "leftColumns", "rightColumns",
        "joinType"} between those operators. Returns each table operator's
        last operator, where its joins attach."""
        def entry(k, v):
            rows, sel = (v, 1.0) if not isinstance(v, tuple) else v
            return {"op": k, "rowCount": int(rows), "selectivity": float(sel)}

        spec = json.dumps({"tables": [entry(k, v) for k, v in tables.items()],
                           "joins": list(joins), "bitsPerKey": bits_per_key, "numHashes": num_hashes,
                           "namePrefix": prefix}).encode()
        L = _abi.lib()
        need = ctypes.c_int64()
        L.gfpdb_plan_predicate_transfer(spec, None, 0, ctypes.byref(need))
        if need.value <= 0:
            _abi.check(L.gfpdb_plan_predicate_transfer(spec, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        _abi.check(L.gfpdb_plan_predicate_transfer(spec, buf, need.value, ctypes.byref(need)))
        out = json.loads(buf.value.decode())
        for op in out["ops"]:
            self._add(op)
        for producer, consumer in out["edges"]:
            self.connect(producer, consumer)
        return out["outputs"]

    def csv_scan(self, name: str, table: str, fields: Sequence[tuple[str, str]], columns: Sequence[str] | None = None,
                 delimiter: str = ",", header: bool = False) -> str:
        """Parse the text held by input `table` (one utf8 value, see
        tupleset.text_table) into the projected `columns`."""
        op = {"type": "CsvScanPOp", "name": name, "table": table,
              "fields": [{"name": n, "type": t} for n, t in fields], "delimiter": delimiter, "header": header}
        if columns:
            op["columns"] = list(columns)
        return self._add(op)

    def project(self, name: str, producer: str, exprs: Sequence[tuple[str, Expr]] = (),
                pairs: Sequence[tuple[str, str]] = ()) -> str:
        """ProjectPOp: pass-through columns renamed (input, output), then one
        column per (name, expression)."""
        self._add({"type": "ProjectPOp", "name": name, "exprs": [{"name": n, "expr": e} for n, e in exprs],
                   "projectColumnNamePairs": [[a, b] for a, b in pairs]})
        self.connect(producer, name)
        return name

    def limit_sort(self, name: str, producer: str, k: int, sort_keys: Sequence[tuple[str, str]],
                   project: Sequence[str] | None = None) -> str:
        """LimitSortPOp: the first k rows by (column, "ASC" | "DESC") keys."""
        op = {"type": "LimitSortPOp", "name": name, "k": k,
              "sortKeys": [{"name": c, "order": o} for c, o in sort_keys]}
        if project is not None:
            op["projectColumnNames"] = list(project)
        self._add(op)
        self.connect(producer, name)
        return name

    def collate(self, name: str, producer: str) -> str:
        self._add({"type": "CollatePOp", "name": name})
        self.connect(producer, name)
        return name

    def to_json(self) -> str:
        return json.dumps({"ops": self.ops}, separators=(",", ":"))


def partial_aggregates(aggregates: Sequence[dict]) -> list[dict]:
    """The first phase of a parallel aggregate
    (PrePToPTransformerUtil::transformAggFunction with a reduce op,
    fpdb-executor/src/physical/transform/PrePToPTransformerUtil.cpp:63-96):
    AVG becomes a SUM and a COUNT into its intermediate columns, the others
    stay as they are."""
    out = []
    for a in aggregates:
        if a["function"].upper() == "AVG":
            out.append({"function": "SUM", "name": "AVG_INTERMEDIATE_SUM_" + a["name"], "expr": a["expr"]})
            out.append({"function": "COUNT", "name": "AVG_INTERMEDIATE_COUNT_" + a["name"], "expr": a["expr"]})
        else:
            out.append(dict(a))
    return out


def reduce_aggregates(aggregates: Sequence[dict]) -> list[dict]:
    """The second phase (PrePToPTransformerUtil::transformAggReduceFunction,
    PrePToPTransformerUtil.cpp:98-124): SUM and COUNT reduce by SUM of the
    partial column, MIN and MAX by themselves, AVG by AVG_REDUCE."""
    out = []
    for a in aggregates:
        fn, name = a["function"].upper(), a["name"]
        if fn == "AVG":
            out.append({"function": "AVG_REDUCE", "name": name})
        else:
            out.append({"function": "SUM" if fn in ("SUM", "COUNT") else fn, "name": name,
                        "expr": {"type": "Column", "columnName": name}})
    return out


def validate(plan: Plan | str) -> None:
    text = plan.to_json() if isinstance(plan, Plan) else plan
    _abi.check(_abi.lib().gfpdb_plan_validate(text.encode()))


def fused(plan: Plan | str) -> dict:
    """The plan after pipeline fusion (gfpdb_plan_fuse, host only): the
    operators a run with "fusePipelines" (the default) executes."""
    text = (plan.to_json() if isinstance(plan, Plan) else plan).encode()
    L = _abi.lib()
    need = ctypes.c_int64()
    rc = L.gfpdb_plan_fuse(text, None, 0, ctypes.byref(need))
    if need.value <= 0:
        _abi.check(rc)
    buf = ctypes.create_string_buffer(need.value)
    _abi.check(L.gfpdb_plan_fuse(text, buf, need.value, ctypes.byref(need)))
    return json.loads(buf.value.decode())


@dataclass
class Result:
    table: Table
    stats: dict


class PreparedInputs:
    """Exported input tables, reusable across executions."""

    def __init__(self, tables: dict[str, Table | DeviceTable | Exported], pinned: bool = False):
        self.names = list(tables)
        self.exported: list[Exported] = []
        for t in tables.values():
            if isinstance(t, Exported):
                self.exported.append(t)
            elif isinstance(t, DeviceTable):
                self.exported.append(t.export())
            else:
                self.exported.append(export_host(t, pinned=pinned))
        n = len(self.names)
        self.c_names = _abi.cstr_array(self.names)
        self.c_schemas = (ctypes.POINTER(_abi.ArrowSchema) * max(1, n))(*[e.schema_ptr for e in self.exported])
        self.c_arrays = (ctypes.POINTER(_abi.ArrowDeviceArray) * max(1, n))(*[e.array_ptr for e in self.exported])


class PreparedPlan:
    """A plan bound to its inputs once (gfpdb_plan_prepare): the library
    validates it once, and with "cudaGraph" every run after the capture is
    one graph replay with no plan lookup or result export; the result is
    read from the prepared plan's host buffers through numpy views that are
    made once per layout. execute() returns copies (the buffers are reused by
    the next run). For a loop that runs one query many times, as a serving
    loop or a benchmark does."""

    MAX_COLUMNS = 256
    NAMES_BYTES = 1 << 16

    def __init__(self, plan: Plan | str, tables: dict | PreparedInputs, result_to_host: bool = True, stream=None):
        if not result_to_host:
            raise ValueError("a prepared plan returns host results")
        self.text = (plan.to_json() if isinstance(plan, Plan) else plan).encode()
        self.inputs = tables if isinstance(tables, PreparedInputs) else PreparedInputs(tables)
        L = _abi.lib()
        self._h = ctypes.c_void_p()
        inp = self.inputs
        _abi.check(L.gfpdb_plan_prepare(self.text, len(inp.names), inp.c_names, inp.c_schemas, inp.c_arrays,
                                        ctypes.byref(self._h)))
        self._run, self._layout, self._free = L.gfpdb_prepared_run, L.gfpdb_prepared_layout, L.gfpdb_prepared_free
        self._launch, self._wait = L.gfpdb_prepared_launch, L.gfpdb_prepared_wait
        self._stats = _abi.ExecStats()
        self._n, self._gen = ctypes.c_int64(), ctypes.c_int64()
        self._args = (self._h, ctypes.byref(self._stats), stream, ctypes.byref(self._n), ctypes.byref(self._gen))
        self._launch_args = (self._h, stream)
        self._wait_args = (self._h, ctypes.byref(self._stats), ctypes.byref(self._n), ctypes.byref(self._gen))
        self._seen_gen = -1
        self._cols = []  # per column: (name, type, values view or None, offsets view or None, data pointer)

    def _refresh(self) -> None:
        cap, nc = ctypes.c_int64(), ctypes.c_int32()
        names = ctypes.create_string_buffer(self.NAMES_BYTES)
        vals = (ctypes.c_void_p * self.MAX_COLUMNS)()
        offs = (ctypes.c_void_p * self.MAX_COLUMNS)()
        _abi.check(self._layout(self._h, self.MAX_COLUMNS, ctypes.byref(cap), ctypes.byref(nc), names, self.NAMES_BYTES,
                                vals, offs))
        parts = names.raw.split(b"\0", 2 * nc.value)
        cols = []
        for i in range(nc.value):
            ty = TYPES[parts[2 * i + 1]]
            name = parts[2 * i].decode()
            if ty == "utf8":
                view = np.frombuffer((ctypes.c_int32 * (cap.value + 1)).from_address(offs[i]), dtype=np.int32)
                cols.append((name, ty, view, vals[i]))
            else:
                dt = np.dtype(NP_TYPES[ty])
                view = np.frombuffer((ctypes.c_char * max(1, cap.value * dt.itemsize)).from_address(vals[i]), dtype=dt)
                cols.append((name, ty, view, None))
        self._cols = cols
        self._seen_gen = self._gen.value

    def execute(self) -> Result:
        _abi.check(self._run(*self._args))
        return self._result()

    def launch(self) -> None:
        """Start a run and return (gfpdb_prepared_launch); wait() finishes
        it. Two prepared plans of one query whose texts differ in
        "graphInstance" can be launched back to back, each waited for while
        the other runs."""
        _abi.check(self._launch(*self._launch_args))

    def wait(self) -> Result:
        _abi.check(self._wait(*self._wait_args))
        return self._result()

    def _result(self) -> Result:
        if self._gen.value != self._seen_gen:
            self._refresh()
        n = self._n.value
        cols = []
        for name, ty, view, data_ptr in self._cols:
            c = Column.__new__(Column)  # the values already have the column's dtype and layout
            c.name, c.type = name, ty
            if ty == "utf8":
                o = view[: n + 1]
                base = int(o[0]) if n >= 0 else 0
                nbytes = int(o[-1]) - base
                data = np.frombuffer((ctypes.c_char * max(1, nbytes)).from_address(data_ptr + base), dtype=np.uint8,
                                     count=nbytes).copy()
                c.values = ((o - base).astype(np.int32), data)
            else:
                c.values = view[:n].copy()
            cols.append(c)
        return Result(Table(cols), {k: getattr(self._stats, k) for k, _ in _abi.ExecStats._fields_})

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._free(self._h)
            self._h = ctypes.c_void_p()


def execute(plan: Plan | str, tables: dict | PreparedInputs, result_to_host: bool = True, stream=None,
            keep_device_result: bool = False):
    """Run a plan; returns Result(table, stats)."""
    text = (plan.to_json() if isinstance(plan, Plan) else plan).encode()
    inputs = tables if isinstance(tables, PreparedInputs) else PreparedInputs(tables)
    s, a = new_output()
    st = _abi.ExecStats()
    _abi.check(_abi.lib().gfpdb_execute_plan(text, len(inputs.names), inputs.c_names, inputs.c_schemas,
                                             inputs.c_arrays, 1 if result_to_host else 0, ctypes.byref(s),
                                             ctypes.byref(a), ctypes.byref(st), stream))
    stats = {k: getattr(st, k) for k, _ in _abi.ExecStats._fields_}
    return Result(import_result(s, a), stats)
