"""Expression builders producing the reference's expression JSON.

The helper names follow the reference's C++ builders in
fpdb-expression-gandiva/include/fpdb/expression/gandiva/ (col, num_lit,
str_lit, lt, lte, gt, gte, eq, neq, and_, or_, not_, plus, minus, times,
divide, cast, in_, isNull) and the node/field names of
Expression::fromJson (fpdb-expression-gandiva/src/Expression.cpp:52-148).
Data types are named ("int32", "int64", "float64", "date32", "boolean",
"utf8") instead of serialised arrow::DataType bytes.
"""

from __future__ import annotations

import json
from typing import Any

Expr = dict


def col(name: str) -> Expr:
    return {"type": "Column", "columnName": name}


def num_lit(value, data_type: str = "int32") -> Expr:
    e = {"type": "NumericLiteral", "dataType": data_type}
    if value is not None:
        e["value"] = value
    return e


def str_lit(value: str) -> Expr:
    return {"type": "StringLiteral", "value": value}


def _bin(kind: str, left: Expr, right: Expr) -> Expr:
    return {"type": kind, "left": left, "right": right}


def lt(l, r):
    return _bin("LessThan", l, r)


def lte(l, r):
    return _bin("LessThanOrEqualTo", l, r)


def gt(l, r):
    return _bin("GreaterThan", l, r)


def gte(l, r):
    return _bin("GreaterThanOrEqualTo", l, r)


def eq(l, r):
    return _bin("EqualTo", l, r)


def neq(l, r):
    return _bin("NotEqualTo", l, r)


def plus(l, r):
    return _bin("Add", l, r)


def minus(l, r):
    return _bin("Subtract", l, r)


def times(l, r):
    return _bin("Multiply", l, r)


def divide(l, r):
    return _bin("Divide", l, r)


def and_(*exprs: Expr) -> Expr:
    if len(exprs) == 1 and isinstance(exprs[0], (list, tuple)):
        exprs = tuple(exprs[0])
    return {"type": "And", "exprs": list(exprs)}


def or_(*exprs: Expr) -> Expr:
    if len(exprs) == 1 and isinstance(exprs[0], (list, tuple)):
        exprs = tuple(exprs[0])
    return {"type": "Or", "exprs": list(exprs)}


def not_(e: Expr) -> Expr:
    return {"type": "Not", "expr": e}


def isNull(e: Expr) -> Expr:
    return {"type": "IsNull", "expr": e}


def cast(e: Expr, data_type: str) -> Expr:
    return {"type": "Cast", "expr": e, "dataType": data_type}


def in_(e: Expr, values: list[Any], data_type: str = "int64") -> Expr:
    return {"type": "In", "expr": e, "values": list(values), "dataType": data_type}


def date_extract(e: Expr, interval: str) -> Expr:
    """DateExtract (interval "Day", "Month" or "Year"): an int64 value."""
    return {"type": "DateExtract", "dateExpr": e, "intervalType": interval}


def date_add(date: Expr, n: Expr, interval: str) -> Expr:
    """DateAdd: date plus n days / months / years (a date32 value)."""
    return {"type": "DateAdd", "left": date, "right": n, "intervalType": interval}


def if_(cond: Expr, then: Expr, otherwise: Expr) -> Expr:
    return {"type": "If", "ifExpr": cond, "thenExpr": then, "elseExpr": otherwise}


def like(e: Expr, pattern: str) -> Expr:
    """SQL LIKE (% any run, _ one character; no escape character)."""
    return {"type": "Like", "left": e, "right": str_lit(pattern)}


def substr(e: Expr, start: int, length: int) -> Expr:
    """SUBSTRING(e FROM start FOR length), 1-based."""
    return {"type": "Substr", "expr": e, "fromLit": num_lit(start, "int64"), "forLit": num_lit(length, "int64")}


def to_json(e: Expr) -> str:
    return json.dumps(e, separators=(",", ":"))
