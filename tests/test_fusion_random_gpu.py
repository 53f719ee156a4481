"""Pipeline fusion on random join trees with data: inner-join trees over 3
to 6 tables, their bloom predicate transfer derived by the planner, run
fused and unfused on the GPU and compared with the oracle's chain of joins
(bloom filters never change an inner join's rows)."""

import json
import random

import numpy as np
import pytest

from flexpushdowndb_gb300 import plan
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops

pytestmark = pytest.mark.gpu


def tree(seed):
    rng = random.Random(seed)
    gen = np.random.default_rng(seed)
    k = rng.randint(3, 6)
    sizes = [rng.choice([300, 2000, 20000, 60000]) for _ in range(k)]
    edges = [(rng.randrange(i), i) for i in range(1, k)]
    children = {i: [c for p, c in edges if p == i] for i in range(k)}
    tables = {}
    for i in range(k):
        cols = [Column(f"t{i}_pk", "int32", gen.permutation(sizes[i]) + 1)]
        for c in children[i]:  # a foreign key into child c: a third of the values miss
            cols.append(Column(f"t{i}_c{c}", "int32", gen.integers(1, int(sizes[c] * 1.5) + 2, sizes[i])))
        tables[f"table{i}"] = Table(cols)
    p = plan.Plan()
    for i in range(k):
        p.scan(f"t{i}", f"table{i}", [c.name for c in tables[f"table{i}"].columns])
    out = p.predicate_transfer({f"t{i}": sizes[i] for i in range(k)},
                               [{"left": f"t{a}", "right": f"t{b}", "leftColumns": [f"t{a}_c{b}"],
                                 "rightColumns": [f"t{b}_pk"], "joinType": "INNER"} for a, b in edges])
    tail = out["t0"]
    for a, b in edges:
        tail = p.hash_join(f"join{b}", out[f"t{b}"], tail, f"t{b}_pk", f"t{a}_c{b}")
    p.collate("collate", tail)
    want = tables["table0"]
    for a, b in edges:
        want = oops.hash_join(tables[f"table{b}"], want, f"t{b}_pk", f"t{a}_c{b}")
    return p, tables, want


@pytest.mark.parametrize("seed", range(12))
def test_random_inner_join_trees(gpu, seed):
    p, tables, want = tree(seed)
    for fuse in (True, False):
        d = json.loads(p.to_json())
        d["fusePipelines"] = fuse
        got = plan.execute(json.dumps(d), tables).table
        assert got.names == want.names
        assert got.sorted_rows() == want.sorted_rows()
