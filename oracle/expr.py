"""Expression evaluation over numpy columns (TEST INFRASTRUCTURE ONLY).

DateExtract / DateAdd follow the proleptic Gregorian calendar over date32
days (DateExtract.cpp, DateAdd.cpp; a day past the end of the new month
becomes its last day); Like is SQL LIKE with % and _ and no escape
character (Like.cpp); Substr is SQL SUBSTRING(s FROM f FOR n) over bytes
(Substr.cpp); If picks per row (If.cpp).

Typing follows the reference (fpdb-expression-gandiva/src/BinaryExpression.cpp:57-102,
castGandivaExprToUpperType): int32 vs int64 operate in int64, int vs double
in double, and same-typed operands keep their type, so int32 * int32 wraps to
int32 as Gandiva's multiply does. Comparisons yield booleans; And / Or / Not
combine them. Integer division truncates toward zero; dividing by zero is an
error, as in Gandiva.
"""

from __future__ import annotations

import calendar as _calendar
import datetime as _dt
import re as _re

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


def _civil(days):
    d = _dt.date(1970, 1, 1) + _dt.timedelta(days=int(days))
    return d.year, d.month, d.day


def _date_add(days: int, n: int, interval: str) -> int:
    if interval == "Day":
        return int(days) + int(n)
    y, m, d = _civil(days)
    months = y * 12 + (m - 1) + (int(n) if interval == "Month" else 12 * int(n))
    ny, nm = divmod(months, 12)
    nm += 1
    dim = _calendar.monthrange(ny, nm)[1]
    return (_dt.date(ny, nm, min(d, dim)) - _dt.date(1970, 1, 1)).days


def _substr(s: str, start: int, length: int) -> str:
    b = s.encode()
    lo, hi = max(start, 1), min(start + length, len(b) + 1)
    return b[lo - 1 : hi - 1].decode() if hi > lo else ""


def _like(s: str, pattern: str) -> bool:
    rx = "".join(".*" if ch == "%" else "." if ch == "_" else _re.escape(ch) for ch in pattern)
    return _re.fullmatch(rx, s, flags=_re.DOTALL) is not None


def value(e: dict, table):
    """Returns (array or scalar, type)."""
    t = e["type"]
    n = table.num_rows
    if t == "DateExtract":
        v, _ = value(e["dateExpr"], table)
        idx = {"Day": 2, "Month": 1, "Year": 0}[e["intervalType"]]
        arr = np.broadcast_to(np.asarray(v), (n,))
        return np.array([_civil(x)[idx] for x in arr.tolist()], dtype=np.int64), "int64"
    if t == "DateAdd":
        a, _ = value(e["left"], table)
        b, _ = value(e["right"], table)
        a = np.broadcast_to(np.asarray(a), (n,)).tolist()
        b = np.broadcast_to(np.asarray(b), (n,)).tolist()
        return np.array([_date_add(x, y, e["intervalType"]) for x, y in zip(a, b)], dtype=np.int32), "date32"
    if t == "If":
        c = predicate(e["ifExpr"], table)
        a, ta = value(e["thenExpr"], table)
        b, tb = value(e["elseExpr"], table)
        rt = "float64" if "float64" in (ta, tb) else (ta if ta == tb else "int64")
        dt = np.float64 if rt == "float64" else np.int64
        r = np.where(c, np.broadcast_to(np.asarray(a).astype(dt), (n,)), np.broadcast_to(np.asarray(b).astype(dt), (n,)))
        return (r.astype(NP[rt]) if rt in NP else r), rt
    if t == "Substr":
        v, _ = value(e["expr"], table)
        f, _ = value(e["fromLit"], table)
        k, _ = value(e["forLit"], table)
        return np.array([_substr(s, int(f), int(k)) for s in v], dtype=object), "utf8"
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
    if t == "Like":
        v, _ = value(e["left"], table)
        pat = e["right"]["value"]
        return np.array([_like(s, pat) for s in v], dtype=bool)
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
