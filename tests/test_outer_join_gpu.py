"""Outer and semi hash joins (the reference's JoinType through
HashJoinArrowKernel's Arrow mapping) on the GPU path against the oracle's
hash_join_typed: through the C ABI (probe batches, then the build side's
rows from finish) and as HashJoinArrowPOps in plans, nulls included."""

import numpy as np
import pytest

from flexpushdowndb_gb300 import GfpdbError, ops, plan
from flexpushdowndb_gb300.expression import col, lt, num_lit, plus
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import ops as oops

pytestmark = pytest.mark.gpu

TYPES = ["INNER", "LEFT", "RIGHT", "FULL", "LEFT_SEMI", "RIGHT_SEMI"]


def sides(nb, np_, seed, bkey="int32", pkey="int32", dup=True):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, max(1, nb * 2), nb) if dup else rng.permutation(max(1, nb * 2))[:nb]
    build = Table([Column("bk", bkey, keys), Column("bv", "int64", rng.integers(-(2**40), 2**40, nb)),
                   Column("bs", "utf8", [f"b{k}" * (1 + k % 3) for k in keys.tolist()])])
    probe = Table([Column("pk", pkey, rng.integers(0, max(1, nb * 2) + 5, np_)),
                   Column("pv", "int32", rng.integers(0, 100, np_)),
                   Column("ps", "utf8", [f"p{i % 7}" for i in range(np_)])])
    return build, probe


def run_abi(build, probe, jt, batches=3, needed=None):
    j = ops.HashJoin("bk", "pk", needed=needed, join_type=jt)
    j.put_build(build)
    j.finalize_build()
    parts = []
    step = max(1, (probe.num_rows + batches - 1) // batches)
    for lo in range(0, max(1, probe.num_rows), step):
        out = j.probe(probe.slice(lo, min(probe.num_rows, lo + step)))
        if out.columns:
            parts.append(out)
    fin = j.finish()
    if fin.columns:
        parts.append(fin)
    rows = sum((p.rows() for p in parts), [])
    return parts, sorted(rows, key=lambda r: tuple((v is None, 0 if v is None else v) for v in r))


@pytest.mark.parametrize("jt", TYPES)
@pytest.mark.parametrize("nb,np_", [(1000, 5000), (0, 100), (50, 0), (20_000, 100_003)])
def test_join_types_match_oracle(gpu, jt, nb, np_):
    build, probe = sides(nb, np_, seed=nb + np_)
    want = oops.hash_join_typed(build, probe, "bk", "pk", jt)
    parts, got = run_abi(build, probe, jt)
    assert got == want.sorted_rows()
    for p in parts:  # columns: probe then build, one side for semi joins
        assert p.names == want.names


@pytest.mark.parametrize("jt", ["LEFT", "RIGHT", "FULL", "RIGHT_SEMI"])
@pytest.mark.parametrize("bkey,pkey", [("int64", "int64"), ("int64", "int32"), ("date32", "date32")])
def test_join_types_key_widths(gpu, jt, bkey, pkey):
    build, probe = sides(3000, 8000, seed=7, bkey=bkey, pkey=pkey)
    want = oops.hash_join_typed(build, probe, "bk", "pk", jt, needed=["pk", "pv", "bk", "bv"])
    _, got = run_abi(build, probe, jt, needed=["pk", "pv", "bk", "bv"])
    assert got == want.sorted_rows()


def test_null_columns_carry_validity(gpu):
    build, probe = sides(100, 300, seed=3)
    parts, _ = run_abi(build, probe, "FULL", batches=1)
    fin = parts[-1]  # unmatched build rows: probe columns null
    assert fin.num_rows > 0
    assert fin.column("pk").valid is not None and not fin.column("pk").valid.any()
    assert fin.column("bk").valid is None


def outer_plan(jt, chunk=0, then=None):
    p = plan.Plan()
    p.scan("b", "build")
    p.scan("p", "probe", chunk_rows=chunk)
    p._add({"type": "HashJoinArrowPOp", "name": "j", "buildProducers": ["b"], "probeProducers": ["p"],
            "buildKey": "bk", "probeKey": "pk", "joinType": jt})
    p.connect("b", "j")
    p.connect("p", "j")
    last = "j"
    if then is not None:
        last = then(p, "j")
    p.collate("collate", last)
    return p


@pytest.mark.parametrize("jt", TYPES)
@pytest.mark.parametrize("chunk", [0, 7000])
def test_join_types_in_plans(gpu, jt, chunk):
    build, probe = sides(5000, 20_000, seed=11)
    got = plan.execute(outer_plan(jt, chunk), {"build": build, "probe": probe}).table
    want = oops.hash_join_typed(build, probe, "bk", "pk", jt)
    assert got.names == want.names
    assert got.sorted_rows() == want.sorted_rows()


@pytest.mark.parametrize("jt", TYPES)
def test_join_types_after_a_selection(gpu, jt):
    """Both sides come from FilterPOps, whose row counts are only known on
    the device: a join that emits its unmatched build rows reads exactly the
    selected build rows, none of the selection's spare capacity."""
    build, probe = sides(6000, 20_000, seed=17)
    p = plan.Plan()
    p.scan("b", "build")
    p.scan("p", "probe")
    p.filter("fb", "b", lt(col("bv"), num_lit(0, "int64")))
    p.filter("fp", "p", lt(col("pv"), num_lit(60, "int32")))
    p._add({"type": "HashJoinArrowPOp", "name": "j", "buildProducers": ["fb"], "probeProducers": ["fp"],
            "buildKey": "bk", "probeKey": "pk", "joinType": jt})
    p.connect("fb", "j")
    p.connect("fp", "j")
    p.collate("collate", "j")
    got = plan.execute(p, {"build": build, "probe": probe}).table
    kb = build["bv"] < 0
    kp = probe["pv"] < 60
    sb = Table([Column(c.name, c.type, c.values[kb] if c.type != "utf8" else [v for v, k in zip(c.to_list(), kb) if k])
                for c in build.columns])
    sp = Table([Column(c.name, c.type, c.values[kp] if c.type != "utf8" else [v for v, k in zip(c.to_list(), kp) if k])
                for c in probe.columns])
    want = oops.hash_join_typed(sb, sp, "bk", "pk", jt)
    assert got.names == want.names
    assert got.sorted_rows() == want.sorted_rows()


def test_nullable_columns_pass_a_projection_but_not_a_group(gpu):
    build, probe = sides(500, 2000, seed=13)
    renamed = plan.execute(outer_plan("LEFT", then=lambda p, j: p.project("proj", j, pairs=[("pv", "x"), ("bk", "k")])),
                           {"build": build, "probe": probe}).table
    want = oops.hash_join_typed(build, probe, "bk", "pk", "LEFT")
    assert renamed.names == ["x", "k"]
    assert renamed.sorted_rows() == sorted([(r[1], r[3]) for r in want.rows()], key=lambda r: tuple((v is None, 0 if v is None else v) for v in r))
    with pytest.raises(GfpdbError) as ei:
        plan.execute(outer_plan("LEFT", then=lambda p, j: p.group("g", j, ["bk"], [ops.aggregate("COUNT", "n")])),
                     {"build": build, "probe": probe})
    assert "nullable" in ei.value.message
    with pytest.raises(GfpdbError) as ei:
        plan.execute(outer_plan("RIGHT", then=lambda p, j: p.project("e", j, exprs=[("y", plus(col("bv"), num_lit(1, "int64")))])),
                     {"build": build, "probe": probe})
    assert "nullable" in ei.value.message


def test_outer_join_needs_one_integer_key(gpu):
    build, probe = sides(10, 10, seed=1)
    j = ops.HashJoin("bs", "ps", join_type="LEFT")
    j.put_build(build)
    with pytest.raises(GfpdbError):
        j.finalize_build()
