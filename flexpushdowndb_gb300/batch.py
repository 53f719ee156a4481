"""Batched star queries through gfpdb_star_batch (see include/gfpdb.h)."""

from __future__ import annotations

import ctypes
import json

from . import _abi
from .plan import PreparedInputs, Result
from .tupleset import import_result, new_output


def star_batch(spec: dict | str, tables, use_graph: bool = True, stream=None) -> Result:
    text = (spec if isinstance(spec, str) else json.dumps(spec)).encode()
    inputs = tables if isinstance(tables, PreparedInputs) else PreparedInputs(tables)
    s, a = new_output()
    st = _abi.ExecStats()
    _abi.check(_abi.lib().gfpdb_star_batch(text, len(inputs.names), inputs.c_names, inputs.c_schemas, inputs.c_arrays,
                                           1 if use_graph else 0, 1, ctypes.byref(s), ctypes.byref(a),
                                           ctypes.byref(st), stream))
    return Result(import_result(s, a), {k: getattr(st, k) for k, _ in _abi.ExecStats._fields_})


def split_by_query(result_table) -> dict[int, list[tuple]]:
    """Rows of a batch result grouped by query_id (query_id column dropped)."""
    out: dict[int, list[tuple]] = {}
    for row in result_table.rows():
        out.setdefault(row[0], []).append(tuple(row[1:]))
    return {q: sorted(v) for q, v in out.items()}


def clear_graph_cache() -> None:
    _abi.check(_abi.lib().gfpdb_graph_cache_clear())


class PreparedBatch:
    """A batched star query bound once to its tables (gfpdb_batch_prepare):
    each run is one graph launch whose result lands in page-locked host
    memory, read here through numpy views made once. launch() / wait() split
    a run so that two prepared copies can be in flight back to back."""

    MAX_COLUMNS = 16
    NAMES_BYTES = 4096

    def __init__(self, spec: dict | str, tables, stream=None):
        import numpy as np

        from .tupleset import NP_TYPES, TYPES

        text = (spec if isinstance(spec, str) else json.dumps(spec)).encode()
        self.inputs = tables if isinstance(tables, PreparedInputs) else PreparedInputs(tables)
        L = _abi.lib()
        self._h = ctypes.c_void_p()
        inp = self.inputs
        _abi.check(L.gfpdb_batch_prepare(text, len(inp.names), inp.c_names, inp.c_schemas, inp.c_arrays,
                                         ctypes.byref(self._h)))
        self._launch, self._wait, self._free = L.gfpdb_batch_launch, L.gfpdb_batch_wait, L.gfpdb_batch_free
        self._stats = _abi.ExecStats()
        self._n = ctypes.c_int64()
        self._stream = stream
        cap, nc = ctypes.c_int64(), ctypes.c_int32()
        names = ctypes.create_string_buffer(self.NAMES_BYTES)
        vals = (ctypes.c_void_p * self.MAX_COLUMNS)()
        _abi.check(L.gfpdb_batch_layout(self._h, self.MAX_COLUMNS, ctypes.byref(cap), ctypes.byref(nc), names,
                                        self.NAMES_BYTES, vals))
        parts = names.raw.split(b"\0", 2 * nc.value)
        self._cols = []
        for i in range(nc.value):
            ty = TYPES[parts[2 * i + 1]]
            dt = np.dtype(NP_TYPES[ty])
            view = np.frombuffer((ctypes.c_char * max(1, cap.value * dt.itemsize)).from_address(vals[i]), dtype=dt)
            self._cols.append((parts[2 * i].decode(), ty, view))

    def launch(self) -> None:
        _abi.check(self._launch(self._h, self._stream))

    def wait(self) -> Result:
        from .tupleset import Column, Table

        _abi.check(self._wait(self._h, ctypes.byref(self._stats), ctypes.byref(self._n)))
        n = self._n.value
        cols = []
        for name, ty, view in self._cols:
            c = Column.__new__(Column)  # the values already have the column's dtype
            c.name, c.type, c.values = name, ty, view[:n].copy()
            cols.append(c)
        return Result(Table(cols), {k: getattr(self._stats, k) for k, _ in _abi.ExecStats._fields_})

    def execute(self) -> Result:
        self.launch()
        return self.wait()

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._free(self._h)
            self._h = ctypes.c_void_p()
