"""Host-side inputs under random and hostile variation, on the CPU: the
predicate compiler (gfpdb_filter_compile, typed random expression trees,
some corrupted) and the predicate-transfer planner (random join-graph
specs with bad names, sizes, types and column lists). Each call returns a
status; none may crash, and what is accepted must be usable (a compiled
filter frees, a planned transfer is valid JSON)."""

import ctypes
import json
import random

import numpy as np

from flexpushdowndb_gb300 import _abi, ops
from flexpushdowndb_gb300.tupleset import Column, Table

CMP = ["LessThan", "LessThanOrEqualTo", "GreaterThan", "GreaterThanOrEqualTo", "EqualTo", "NotEqualTo"]


class ExprGen:
    def __init__(self, seed, max_depth=8):
        self.rng = random.Random(seed)
        self.max_depth = max_depth

    def lit(self):
        r = self.rng
        ty = r.choice(["int32", "int64", "float64"])
        v = r.choice([0, 1, -3, 7, 2**33]) if ty != "float64" else r.choice([0.5, -2.0, 1e9])
        return {"type": "NumericLiteral", "dataType": ty, "value": v}

    def num(self, d):
        r = self.rng
        x = r.random()
        if d >= self.max_depth or x < 0.3:
            return r.choice([{"type": "Column", "name": r.choice(["a", "b", "f"])}, self.lit()])
        if x < 0.75:
            return {"type": r.choice(["Add", "Subtract", "Multiply", "Divide"]), "left": self.num(d + 1),
                    "right": self.num(d + 1)}
        if x < 0.85:
            return {"type": "Cast", "expr": self.num(d + 1), "dataType": r.choice(["int64", "float64", "int32"])}
        if x < 0.92:
            return {"type": "If", "ifExpr": self.boolean(d + 1), "thenExpr": self.num(d + 1),
                    "elseExpr": self.num(d + 1)}
        return {"type": "DateExtract", "dateExpr": self.date(d + 1), "intervalType": r.choice(["Year", "Month", "Day"])}

    def date(self, d):
        if d >= self.max_depth or self.rng.random() < 0.6:
            return {"type": "Column", "name": "d"}
        return {"type": "DateAdd", "left": self.date(d + 1), "right": self.num(d + 1),
                "intervalType": self.rng.choice(["Day", "Month", "Year"])}

    def string(self, d):
        r = self.rng
        if d >= self.max_depth or r.random() < 0.7:
            return {"type": "Column", "name": "s"}
        return {"type": "Substr", "expr": self.string(d + 1),
                "fromLit": {"type": "NumericLiteral", "dataType": "int64", "value": r.randint(-2, 4)},
                "forLit": {"type": "NumericLiteral", "dataType": "int64", "value": r.randint(-1, 4)}}

    def boolean(self, d):
        r = self.rng
        x = r.random()
        if d >= self.max_depth or x < 0.4:
            c = r.random()
            if c < 0.6:
                return {"type": r.choice(CMP), "left": self.num(d + 1), "right": self.num(d + 1)}
            if c < 0.75:
                return {"type": "EqualTo", "left": self.string(d + 1),
                        "right": {"type": "StringLiteral", "value": r.choice(["x", "", "xy"])}}
            if c < 0.85:
                return {"type": "Like", "left": self.string(d + 1),
                        "right": {"type": "StringLiteral", "value": r.choice(["x%", "%", "_", "%y%", ""])}}
            if c < 0.93:
                return {"type": "In", "expr": self.num(d + 1),
                        "values": [r.randint(-5, 5) for _ in range(r.randint(0, 5))], "dataType": "int64"}
            return {"type": "IsNull", "expr": self.num(d + 1)}
        if x < 0.8:
            return {"type": r.choice(["And", "Or"]), "exprs": [self.boolean(d + 1) for _ in range(r.randint(1, 4))]}
        return {"type": "Not", "expr": self.boolean(d + 1)}

    def corrupt(self, e):
        r = self.rng
        if isinstance(e, dict):
            if r.random() < 0.05 and e:
                k = r.choice(list(e))
                if r.random() < 0.5:
                    e.pop(k)
                else:
                    e[k] = r.choice([self.num(self.max_depth), self.string(self.max_depth),
                                     self.boolean(self.max_depth), None, 3, "x", []])
                return e
            for k in list(e):
                self.corrupt(e[k])
        elif isinstance(e, list):
            for x in e:
                self.corrupt(x)
        return e


def test_random_predicates_compile_or_are_refused():
    t = Table([Column("a", "int32", np.arange(4)), Column("b", "int64", np.arange(4)),
               Column("f", "float64", np.arange(4.0)), Column("d", "date32", np.arange(4)),
               Column("s", "utf8", ["x", "y", "z", "w"])])
    ex = ops._export(t)
    L = _abi.lib()
    gen = ExprGen(31)
    h = ctypes.c_void_p()
    compiled = refused = 0
    for _ in range(1500):
        e = gen.boolean(0)
        if gen.rng.random() < 0.3:
            e = gen.corrupt(e)
        text = json.dumps(e).encode()
        if gen.rng.random() < 0.1:  # broken JSON too
            b = bytearray(text)
            b[gen.rng.randrange(len(b))] = gen.rng.choice(b'{}[]",:0123456789')
            text = bytes(b)
        if L.gfpdb_filter_compile(text, ex.schema_ptr, ctypes.byref(h)) == 0:
            L.gfpdb_filter_free(h)
            compiled += 1
        else:
            refused += 1
    assert compiled > 100 and refused > 100


def test_random_transfer_specs_plan_or_are_refused():
    L = _abi.lib()
    rng = random.Random(11)
    types = ["INNER", "LEFT", "RIGHT", "FULL", "LEFT_SEMI", "RIGHT_SEMI", "BOGUS"]
    need = ctypes.c_int64()
    planned = refused = 0
    for _ in range(1500):
        names = [rng.choice(["a", "b", "c", "d", "e", "f", 'q"x', "", "a"]) for _ in range(rng.randint(0, 8))]
        tables = [{"op": n, "rowCount": rng.choice([0, 1, 10, 10**6, -5, 2**62]),
                   "selectivity": rng.choice([0.0, 0.5, 1.0, -1.0, 1e300])} for n in names]
        joins = []
        for _ in range(rng.randint(0, 12)):
            pool = names + ["zz"]
            nc = rng.randint(0, 3)
            joins.append({"left": rng.choice(pool), "right": rng.choice(pool),
                          "leftColumns": [f"c{i}" for i in range(nc)],
                          "rightColumns": [f"d{i}" for i in range(rng.choice([nc, nc, nc + 1]))],
                          "joinType": rng.choice(types)})
        spec = {"tables": tables, "joins": joins, "bitsPerKey": rng.choice([1, 10, 0, 100]),
                "numHashes": rng.choice([1, 3, 9]), "namePrefix": rng.choice(["pt", "", 'x"y'])}
        if rng.random() < 0.1:
            del spec["tables"]
        text = json.dumps(spec).encode()
        rc = L.gfpdb_plan_predicate_transfer(text, None, 0, ctypes.byref(need))
        if need.value > 0 and rc != 0:
            buf = ctypes.create_string_buffer(need.value)
            rc = L.gfpdb_plan_predicate_transfer(text, buf, need.value, ctypes.byref(need))
            if rc == 0:
                out = json.loads(buf.value.decode())
                assert set(out) == {"ops", "edges", "outputs"}
        if rc == 0:
            planned += 1
        else:
            refused += 1
    assert planned > 50 and refused > 50


def test_random_group_specs_compile_or_are_refused():
    L = _abi.lib()
    rng = random.Random(5)
    fns = ["SUM", "COUNT", "AVG", "MIN", "MAX", "AVG_REDUCE", "sum", "BOGUS", "", None]

    def expr():
        return rng.choice([{"type": "Column", "name": rng.choice(["a", "b", ""])},
                           {"type": "Multiply", "left": {"type": "Column", "name": "a"},
                            "right": {"type": "Column", "name": "b"}},
                           {"type": "NumericLiteral", "dataType": "int64", "value": 3}, None, 5, "x",
                           {"type": "Bogus"}])

    h = ctypes.c_void_p()
    made = refused = 0
    for _ in range(1500):
        aggs = []
        for _ in range(rng.randint(0, 9)):
            a = {"function": rng.choice(fns), "name": rng.choice(["s", "c", "", 's"q'])}
            if rng.random() < 0.7:
                a["expr"] = expr()
            if rng.random() < 0.1:
                a = rng.choice([None, 3, "x", []])
            aggs.append(a)
        spec = {"groupColumnNames": [rng.choice(["a", "b", "c", ""]) for _ in range(rng.randint(0, 10))],
                "aggregates": aggs}
        if rng.random() < 0.1:
            spec.pop(rng.choice(list(spec)))
        if rng.random() < 0.1:
            spec["groupsHint"] = rng.choice([-1, 0, 2**62, "x"])
        if L.gfpdb_group_create(json.dumps(spec).encode(), ctypes.byref(h)) == 0:
            L.gfpdb_group_free(h)
            made += 1
        else:
            refused += 1
    assert made > 50 and refused > 50
