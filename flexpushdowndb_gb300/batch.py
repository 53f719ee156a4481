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
