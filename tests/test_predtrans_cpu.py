"""The predicate-transfer planner (gfpdb_plan_predicate_transfer,
SmallToLargePredTransOrder) on CPU: the filters a join graph gets, their
order and placement, the directions outer joins block, cycles."""

import pytest

from flexpushdowndb_gb300 import _abi, plan


def star_joins():
    dims = {"d1": 1000, "d2": 200, "d3": 500, "d4": 50}
    tables = dict(dims, fact=6_000_000)
    # joins written fact-first: the planner orients them small -> large
    joins = [{"left": "fact", "right": d, "leftColumns": [f"fk{d[1]}"], "rightColumns": [f"{d}_pk"],
              "joinType": "INNER"} for d in dims]
    return tables, joins


def ops_of(p, kind):
    return [o for o in p.ops if o["type"] == kind]


def test_star_graph_filters_small_to_large():
    p = plan.Plan()
    tables, joins = star_joins()
    for t in tables:
        p.scan(t, t)
    out = p.predicate_transfer(tables, joins)
    creates, uses = ops_of(p, "BloomFilterCreatePOp"), ops_of(p, "BloomFilterUsePOp")
    assert len(creates) == len(uses) == 8  # a forward and a backward filter per join
    # forward uses chain on the fact, smallest dimension first
    chain, op = [], "fact"
    while True:
        nxt = [c for c in p.op(op).get("consumers", []) if c.endswith(tuple(f"use_fw{k}" for k in range(8)))]
        if not nxt:
            break
        op = nxt[0]
        chain.append(p.op(op)["bloomFilterColumn"])
    assert chain == ["fk4", "fk2", "fk3", "fk1"]
    # backward filters are created on the fact after every forward use, used on the dimensions
    last_fw = op
    bw_creates = [c for c in creates if "_bw" in c["name"]]
    assert all(c["name"] in p.op(last_fw)["consumers"] for c in bw_creates)
    assert out["fact"] == last_fw
    for d in ("d1", "d2", "d3", "d4"):
        assert "_bf_use_bw" in out[d]
        assert p.op(out[d])["bloomFilterColumn"] == f"{d}_pk"


def chain_graph(join_type):
    p = plan.Plan()
    tables = {"a": 10, "b": 1000, "c": 100_000}
    for t in tables:
        p.scan(t, t)
    joins = [{"left": "a", "right": "b", "leftColumns": ["ak"], "rightColumns": ["b_a"], "joinType": join_type},
             {"left": "b", "right": "c", "leftColumns": ["bk"], "rightColumns": ["c_b"], "joinType": "INNER"}]
    return p, tables, joins


@pytest.mark.parametrize("jt,fw,bw", [("INNER", 2, 2), ("LEFT", 2, 1), ("RIGHT", 1, 2), ("FULL", 1, 1),
                                      ("LEFT_SEMI", 2, 2), ("RIGHT_SEMI", 2, 2)])
def test_outer_joins_block_directions(jt, fw, bw):
    p, tables, joins = chain_graph(jt)
    p.predicate_transfer(tables, joins)
    names = [o["name"] for o in ops_of(p, "BloomFilterCreatePOp")]
    assert sum("_fw" in n for n in names) == fw
    assert sum("_bw" in n for n in names) == bw


def test_transitive_forward_order():
    """a's filter reaches c through b: b's filter on c is created after a's
    filter was applied to b."""
    p, tables, joins = chain_graph("INNER")
    out = p.predicate_transfer(tables, joins)
    fw_use_b = next(o for o in ops_of(p, "BloomFilterUsePOp") if o["bloomFilterColumn"] == "b_a")
    create_on_b = next(o for o in ops_of(p, "BloomFilterCreatePOp") if o["bloomFilterColumn"] == "bk")
    assert create_on_b["name"] in fw_use_b["consumers"]
    assert out["c"].startswith("pt_bf_use")


def test_orientation_by_row_count_reverses_join_type():
    p = plan.Plan()
    tables = {"big": 10_000, "small": 10}
    for t in tables:
        p.scan(t, t)
    # LEFT join written big-first: small-first it is a RIGHT join (no forward filter)
    p.predicate_transfer(tables, [{"left": "big", "right": "small", "leftColumns": ["x"], "rightColumns": ["y"],
                                   "joinType": "LEFT"}])
    names = [o["name"] for o in ops_of(p, "BloomFilterCreatePOp")]
    assert names == ["pt_bf_create_bw0"]


def test_cycles_and_bad_specs_fail():
    def scans(tables):
        p = plan.Plan()
        for t in tables:
            p.scan(t, t)
        return p

    cyc = [{"left": "a", "right": "b", "leftColumns": ["x"], "rightColumns": ["x"]},
           {"left": "b", "right": "c", "leftColumns": ["y"], "rightColumns": ["y"]},
           {"left": "c", "right": "a", "leftColumns": ["z"], "rightColumns": ["z"]}]
    # row counts orient c -> a as a -> c: no cycle
    tables = {"a": 10, "b": 20, "c": 30}
    scans(tables).predicate_transfer(tables, cyc)
    # equal row counts keep the written directions: a -> b -> c -> a
    tables = {"a": 10, "b": 10, "c": 10}
    with pytest.raises(_abi.GfpdbError) as ei:
        scans(tables).predicate_transfer(tables, cyc)
    assert "cycle" in ei.value.message
    with pytest.raises(_abi.GfpdbError) as ei:
        plan.Plan().predicate_transfer({"a": 10}, [{"left": "a", "right": "zz", "leftColumns": ["x"],
                                                   "rightColumns": ["x"]}])
    assert "not listed" in ei.value.message


def test_planned_star_query_matches_the_written_one():
    """The planner, given the star query's join graph, places the filters the
    hand-written star plan has: forward uses on the fact in the written probe
    order (most selective first), a backward filter from the fact's last
    forward use to every dimension."""
    from flexpushdowndb_gb300 import workloads

    p = workloads.star_plan_planned()
    plan.validate(p)
    fw_cols, op = [], "scan_fact"
    while True:
        nxt = [c for c in p.op(op).get("consumers", []) if "_bf_use_fw" in c]
        if not nxt:
            break
        op = nxt[0]
        fw_cols.append(p.op(op)["bloomFilterColumn"])
    written = workloads.star_plan()
    want = [o["bloomFilterColumn"] for o in written.ops if o["name"].startswith("bf_fwd_use_")]
    assert fw_cols == want == ["fk2", "fk3", "fk4", "fk1"]
    bw = sorted(o["bloomFilterColumn"] for o in p.ops if "_bf_use_bw" in o["name"])
    assert bw == ["d1_pk", "d2_pk", "d3_pk", "d4_pk"]
    for o in p.ops:
        if "_bf_create_bw" in o["name"]:
            assert o["name"] in p.op(op)["consumers"]
