"""Expression evaluation over numpy columns (TEST INFRASTRUCTURE ONLY).

Typing follows the reference (fpdb-expression-gandiva/src/BinaryExpression.cpp:57-102,
castGandivaExprToUpperType): int32 vs int64 operate in int64, int vs double
in double, and same-typed operands keep their type, so int32 * int32 wraps to
int32 as Gandiva's multiply does. Comparisons yield booleans; And / Or / Not
combine them. Integer division truncates toward zero; dividing by zero is an
error, as in Gandiva.
"""

from __future__ import annotations

import numpy as np

INT_TYPES = ("int32", "int64", "date32")
NP = {"int32": np.int32, "int64": np.int64, "date32": np.int32, "float64": np.float64}


class OracleError(ValueError):
    pass


def _column(table, name):
    try:
        c = table.column(name)
    except KeyError:
        raise OracleError(f"column '{name}' not found")
    if c.type == "utf8":
        return np.array(c.to_list(), dtype=object), "utf8"
    return c.values, c.type


def _promote(ta: str, tb: str) -> str:
    if "float64" in (ta, tb):
        return "float64"
    if "int64" in (ta, tb):
        return "int64"
    return "int32"


def value(e: dict, table):
    """Returns (array or scalar, type)."""
    t = e["type"]
    if t == "Column":
        return _column(table, e.get("columnName", e.get("name")))
    if t == "NumericLiteral":
        dt = e["dataType"]
        if dt == "boolean":
            return bool(e["value"]), "boolean"
        return NP[dt](e["value"]), dt
    if t == "StringLiteral":
        return e["value"], "utf8"
    if t == "Cast":
        v, vt = value(e["expr"], table)
        to = e["dataType"]
        if to == "float64":
            return np.asarray(v).astype(np.float64), "float64"
        if vt == "float64":
            return np.trunc(np.asarray(v, dtype=np.float64)).astype(np.int64).astype(NP[to]), to
        return np.asarray(v).astype(np.int64).astype(NP[to]), to
    if t in ("Add", "Subtract", "Multiply", "Divide"):
        a, ta = value(e["left"], table)
        b, tb = value(e["right"], table)
        rt = _promote(ta, tb)
        wide = np.float64 if rt == "float64" else np.int64
        a = np.asarray(a).astype(wide)
        b = np.asarray(b).astype(wide)
        with np.errstate(over="ignore"):
            if t == "Add":
                r = a + b
            elif t == "Subtract":
                r = a - b
            elif t == "Multiply":
                r = a * b
            else:
                if rt == "float64":
                    r = a / b
                else:
                    if np.any(b == 0):
                        raise OracleError("divide by zero")
                    q = np.abs(a) // np.abs(b)
                    r = np.where((a < 0) != (b < 0), -q, q)
        if rt == "int32":
            r = np.asarray(r).astype(np.int64).astype(np.int32)  # wraps like int32 arithmetic
        return r, rt
    raise OracleError(f"not a value expression: {t}")


def predicate(e: dict, table) -> np.ndarray:
    n = table.num_rows
    t = e["type"]
    if t == "And":
        out = np.ones(n, dtype=bool)
        for k in e["exprs"]:
            out &= predicate(k, table)
        return out
    if t == "Or":
        out = np.zeros(n, dtype=bool)
        for k in e["exprs"]:
            out |= predicate(k, table)
        return out
    if t == "Not":
        return ~predicate(e["expr"], table)
    if t == "IsNull":
        return np.zeros(n, dtype=bool)  # inputs carry no nulls
    if t == "NumericLiteral" and e.get("dataType") == "boolean":
        return np.full(n, bool(e["value"]))
    if t == "In":
        v, vt = value(e["expr"], table)
        if vt == "utf8":
            s = set(e["values"])
            return np.array([x in s for x in v], dtype=bool)
        vals = np.array(e["values"], dtype=np.float64 if vt == "float64" or e.get("dataType") == "float64" else np.int64)
        return np.isin(np.asarray(v).astype(vals.dtype), vals)
    ops = {"LessThan": np.less, "LessThanOrEqualTo": np.less_equal, "GreaterThan": np.greater,
           "GreaterThanOrEqualTo": np.greater_equal, "EqualTo": np.equal, "NotEqualTo": np.not_equal}
    if t in ops:
        a, ta = value(e["left"], table)
        b, tb = value(e["right"], table)
        if "utf8" in (ta, tb):
            if t not in ("EqualTo", "NotEqualTo"):
                raise OracleError("only = and != compare strings")
            r = np.asarray(a, dtype=object) == np.asarray(b, dtype=object)
            r = np.broadcast_to(r, (n,)).copy()
            return r if t == "EqualTo" else ~r
        ct = np.float64 if "float64" in (ta, tb) else np.int64
        r = ops[t](np.asarray(a).astype(ct), np.asarray(b).astype(ct))
        return np.broadcast_to(r, (n,)).copy()
    raise OracleError(f"not a boolean expression: {t}")
