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

from . import _abi
from .expression import Expr
from .tupleset import DeviceTable, Exported, ResultReader, Table, export_host, import_result, new_output


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

    def scan(self, name: str, table: str, columns: Sequence[str] | None = None, chunk_rows: int = 0) -> str:
        op = {"type": "TableScanPOp", "name": name, "table": table}
        if columns:
            op["columns"] = list(columns)
        if chunk_rows:
            op["chunkRows"] = chunk_rows
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

    def hash_join(self, name: str, build: str, probe: str, build_key: str, probe_key: str,
                  project: Sequence[str] | None = None, load_factor: float = 0.5) -> str:
        op = {"type": "HashJoinArrowPOp", "name": name, "buildProducers": [build], "probeProducers": [probe],
              "buildKey": build_key, "probeKey": probe_key, "joinType": "INNER", "loadFactor": load_factor}
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

    def csv_scan(self, name: str, table: str, fields: Sequence[tuple[str, str]], columns: Sequence[str] | None = None,
                 delimiter: str = ",", header: bool = False) -> str:
        """Parse the text held by input `table` (one utf8 value, see
        tupleset.text_table) into the projected `columns`."""
        op = {"type": "CsvScanPOp", "name": name, "table": table,
              "fields": [{"name": n, "type": t} for n, t in fields], "delimiter": delimiter, "header": header}
        if columns:
            op["columns"] = list(columns)
        return self._add(op)

    def collate(self, name: str, producer: str) -> str:
        self._add({"type": "CollatePOp", "name": name})
        self.connect(producer, name)
        return name

    def to_json(self) -> str:
        return json.dumps({"ops": self.ops}, separators=(",", ":"))


def validate(plan: Plan | str) -> None:
    text = plan.to_json() if isinstance(plan, Plan) else plan
    _abi.check(_abi.lib().gfpdb_plan_validate(text.encode()))


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
    """A plan bound to its inputs once: the encoded plan text, the exported
    inputs and the call's argument structures are made here and reused, so
    execute() does the least host work per call (a loop that runs one query
    many times, as a serving loop or a benchmark does)."""

    def __init__(self, plan: Plan | str, tables: dict | PreparedInputs, result_to_host: bool = True, stream=None):
        self.text = (plan.to_json() if isinstance(plan, Plan) else plan).encode()
        self.inputs = tables if isinstance(tables, PreparedInputs) else PreparedInputs(tables)
        self.result_to_host = 1 if result_to_host else 0
        self.stream = stream
        self._stats = _abi.ExecStats()
        self._fn = _abi.lib().gfpdb_execute_plan
        self._reader = ResultReader()
        self._s, self._a = new_output()  # reused: the reader releases them after every call
        inp = self.inputs
        self._args = (self.text, len(inp.names), inp.c_names, inp.c_schemas, inp.c_arrays, self.result_to_host,
                      ctypes.byref(self._s), ctypes.byref(self._a), ctypes.byref(self._stats), stream)

    def execute(self) -> Result:
        _abi.check(self._fn(*self._args))
        table = self._reader.read(self._s, self._a)
        return Result(table, {k: getattr(self._stats, k) for k, _ in _abi.ExecStats._fields_})


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
