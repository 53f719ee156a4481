"""Pipeline fusion (gfpdb_plan_fuse) on CPU: which operators a plan's run
executes. Bloom selections chained on one input merge; a bloom selection
feeding only an inner join's build side, on the join key, is folded into the
join build; chains of inner joins merge; everything else is left alone."""

import json

import pytest

from flexpushdowndb_gb300 import GfpdbError, plan, workloads


def by_name(fused):
    return {o["name"]: o for o in fused["ops"]}


def test_star_backward_filters_fold_into_join_chain():
    f = plan.fused(workloads.star_plan())
    ops = by_name(f)
    assert len(f["ops"]) == 18
    assert [o["name"] for o in f["ops"] if o["type"] == "BloomFilterUsePOp"] == ["bf_fwd_use_fk1"]
    chain = ops["join_d4"]
    assert chain["type"] == "HashJoinChainPOp"
    for i, j in enumerate(chain["joins"], start=1):
        assert j["name"] == f"join_d{i}"
        # the dimension's rows come straight from the forward filter's creator
        assert j["buildProducers"] == [f"bf_fwd_create_d{i}"]
        # each filter is known by the creator it came from
        assert j["buildFilters"] == [{"column": f"d{i}_pk", "creator": f"bf_bwd_create_fk{i}"}]
    # the backward creators merged into the last one, which both feeds the
    # chain's probe side and sends it the filters: its rows go by its data
    # consumers
    assert ops["bf_bwd_create_fk4"]["bloomFilterUsePOps"] == ["join_d4"]
    assert ops["bf_bwd_create_fk4"]["dataConsumers"] == ["join_d4"]
    assert chain["probeProducers"] == ["bf_bwd_create_fk4"]
    plan.validate(json.dumps(f))


def test_planned_star_fuses_like_the_written_one():
    f = plan.fused(workloads.star_plan_planned())
    assert len(f["ops"]) == 18
    uses = [o for o in f["ops"] if o["type"] == "BloomFilterUsePOp"]
    assert len(uses) == 1 and len(uses[0]["creators"]) == 4
    chain = by_name(f)["join_d4"]
    assert [j["buildProducers"] for j in chain["joins"]] == [[f"filter_d{i}"] for i in range(1, 5)]
    assert all(len(j["buildFilters"]) == 1 for j in chain["joins"])


def two_table(join_type="INNER", use_column="d_pk", extra_consumer=False, probe_side=False):
    p = plan.Plan()
    p.scan("scan_d", "dim", ["d_pk", "d_v"])
    p.scan("scan_f", "fact", ["fk", "x"])
    c = p.bloom_create("bw_create", "scan_f", "fk")
    u = p.bloom_use("bw_use", "scan_d", c, use_column)
    if probe_side:
        p.hash_join("join", "bw_create", u, "fk", "d_pk", ["x", "d_v"], join_type=join_type)
    else:
        p.hash_join("join", u, c, "d_pk", "fk", ["x", "d_v"], join_type=join_type)
    p.collate("collate", "join")
    if extra_consumer:
        p.collate("collate2", u)
    return p


def test_single_join_folds_its_build_filter():
    f = plan.fused(two_table())
    ops = by_name(f)
    assert "bw_use" not in ops
    j = ops["join"]
    assert j["type"] == "HashJoinArrowPOp"
    assert j["buildProducers"] == ["scan_d"]
    assert j["buildFilters"] == [{"column": "d_pk", "creator": "bw_create"}]
    assert ops["bw_create"]["dataConsumers"] == ["join"]
    assert ops["bw_create"]["bloomFilterUsePOps"] == ["join"]
    assert ops["scan_d"]["consumers"] == ["join"]


@pytest.mark.parametrize("case", ["left", "full", "left_semi", "other_column", "two_consumers", "probe_side"])
def test_build_filter_not_folded(case):
    kw = {"left": dict(join_type="LEFT"), "full": dict(join_type="FULL"),
          "left_semi": dict(join_type="LEFT_SEMI"), "other_column": dict(use_column="d_v"),
          "two_consumers": dict(extra_consumer=True), "probe_side": dict(probe_side=True)}[case]
    f = plan.fused(two_table(**kw))
    ops = by_name(f)
    assert "bw_use" in ops
    assert "buildFilters" not in ops["join"]


def test_fuse_keeps_plans_without_candidates():
    p = plan.Plan()
    p.scan("s", "t", ["a"])
    p.collate("c", "s")
    assert plan.fused(p)["ops"] == json.loads(p.to_json())["ops"]


def test_creator_chain_and_siblings_merge():
    f = by_name(plan.fused(workloads.star_plan()))
    c = f["bf_bwd_create_fk4"]
    assert [x["origin"] for x in c["filters"]] == [f"bf_bwd_create_fk{i}" for i in range(1, 5)]
    assert [x["bloomFilterColumn"] for x in c["filters"]] == [f"fk{i}" for i in range(1, 5)]
    assert all(x["bloomFilterUsePOps"] == ["join_d4"] for x in c["filters"])
    assert c["dataConsumers"] == ["join_d4"]
    for i in range(1, 4):
        assert f"bf_bwd_create_fk{i}" not in f
    # the forward creators read different dimensions: left alone
    assert all(f"bf_fwd_create_d{i}" in f for i in range(1, 5))
    # the planner's backward creators are siblings on the fact's last use
    g = plan.fused(workloads.star_plan_planned())
    creators = [o for o in g["ops"] if o["type"] == "BloomFilterCreatePOp" and "filters" in o]
    assert len(creators) == 1 and len(creators[0]["filters"]) == 4
    assert len(g["ops"]) == 18


def test_creator_merge_limit():
    p = plan.Plan()
    p.scan("s", "t", ["k"])
    p.scan("x", "u", ["k"])
    prev, tail = "s", "x"
    for i in range(10):
        prev = p.bloom_create(f"c{i}", prev, "k")
        tail = p.bloom_use(f"u{i}", tail, prev, "k")
    p.collate("collate", tail)
    f = plan.fused(p)
    sizes = sorted(len(o.get("filters", [o])) for o in f["ops"] if o["type"] == "BloomFilterCreatePOp")
    assert sizes == [2, 8]


def test_two_filters_fold_into_one_join_build():
    p = plan.Plan()
    p.scan("scan_d", "dim", ["d_pk"])
    p.scan("scan_f", "fact", ["fk"])
    p.scan("scan_g", "fact2", ["gk"])
    c1 = p.bloom_create("bw1", "scan_f", "fk")
    c2 = p.bloom_create("bw2", "scan_g", "gk")
    u1 = p.bloom_use("use1", "scan_d", c1, "d_pk")
    u2 = p.bloom_use("use2", u1, c2, "d_pk")
    p.hash_join("join", u2, c1, "d_pk", "fk")
    p.collate("collate", "join")
    ops = by_name(plan.fused(p))
    assert "use1" not in ops and "use2" not in ops
    assert ops["join"]["buildProducers"] == ["scan_d"]
    assert ops["join"]["buildFilters"] == [{"column": "d_pk", "creator": "bw1"}, {"column": "d_pk", "creator": "bw2"}]
    # different rows: the two creators stay apart
    assert "filters" not in ops["bw1"] and "filters" not in ops["bw2"]
    assert ops["bw1"]["dataConsumers"] == ["join"] and ops["bw2"]["dataConsumers"] == []


@pytest.mark.parametrize("make", ["star", "planned", "two_table", "two_filters"])
def test_fusion_is_idempotent(make):
    """Fusing a fused plan changes nothing, and the fused plan is valid JSON
    the plan checker accepts."""
    if make == "star":
        text = workloads.star_plan().to_json()
    elif make == "planned":
        text = workloads.star_plan_planned().to_json()
    elif make == "two_table":
        text = two_table().to_json()
    else:
        p = plan.Plan()
        p.scan("scan_d", "dim", ["d_pk"])
        p.scan("scan_f", "fact", ["fk"])
        p.scan("scan_g", "fact2", ["gk"])
        c1 = p.bloom_create("bw1", "scan_f", "fk")
        c2 = p.bloom_create("bw2", "scan_g", "gk")
        u2 = p.bloom_use("use2", p.bloom_use("use1", "scan_d", c1, "d_pk"), c2, "d_pk")
        p.hash_join("join", u2, c1, "d_pk", "fk")
        p.collate("collate", "join")
        text = p.to_json()
    once = plan.fused(text)
    twice = plan.fused(json.dumps(once))
    assert twice == once
    plan.validate(json.dumps(once))


def test_plan_builder_join_types_and_key_lists():
    p = plan.Plan()
    p.scan("a", "ta", ["k1", "k2", "v"])
    p.scan("b", "tb", ["j1", "j2", "w"])
    p.hash_join("j", "a", "b", ["k1", "k2"], ["j1", "j2"], ["v", "w", "k1"])
    p.hash_join("l", "j", "b", "k1", "j1", ["v", "w"], join_type="LEFT")
    p.collate("c", "l")
    op = p.op("j")
    assert op["buildKeys"] == ["k1", "k2"] and op["probeKeys"] == ["j1", "j2"] and op["joinType"] == "INNER"
    assert "buildKey" not in op
    assert p.op("l")["joinType"] == "LEFT" and p.op("l")["buildKey"] == "k1"
    plan.validate(p)
    with pytest.raises(ValueError):
        plan.Plan().hash_join("x", "a", "b", ["k1", "k2"], ["j1"])
    # outer and semi joins take one key column per side
    q = plan.Plan()
    q.scan("a", "ta", ["k1", "k2"])
    q.scan("b", "tb", ["j1", "j2"])
    q.hash_join("j", "a", "b", ["k1", "k2"], ["j1", "j2"], join_type="LEFT")
    q.collate("c", "j")
    with pytest.raises(GfpdbError):
        plan.validate(q)


def random_join_tree(seed):
    """A random join tree over 3-6 tables, planned by the predicate-transfer
    planner, then joined child after child into the first table's rows."""
    import random

    rng = random.Random(seed)
    k = rng.randint(3, 6)
    types = ["INNER", "INNER", "INNER", "LEFT", "RIGHT", "FULL", "LEFT_SEMI", "RIGHT_SEMI"]
    p = plan.Plan()
    tables, joins, edges = {}, [], []
    for i in range(k):
        cols = [f"t{i}_pk"] + [f"t{i}_c{j}" for j in range(i + 1, k)]
        p.scan(f"t{i}", f"table{i}", cols)
        tables[f"t{i}"] = (rng.choice([50, 500, 5000, 50000, 500000]), rng.choice([1.0, 0.5, 0.1]))
    for i in range(1, k):
        parent = rng.randrange(i)
        jt = rng.choice(types)
        edges.append((parent, i, jt))
        joins.append({"left": f"t{parent}", "right": f"t{i}", "leftColumns": [f"t{parent}_c{i}"],
                      "rightColumns": [f"t{i}_pk"], "joinType": jt})
    out = p.predicate_transfer(tables, joins)
    tail = out["t0"]
    for parent, child, jt in edges:
        name = f"join{child}"
        p.hash_join(name, out[f"t{child}"], tail, f"t{child}_pk", f"t{parent}_c{child}", join_type=jt)
        tail = name
    p.collate("collate", tail)
    return p


@pytest.mark.parametrize("seed", range(40))
def test_fusion_invariants_on_random_join_trees(seed):
    p = random_join_tree(seed)
    plan.validate(p)
    f = plan.fused(p)
    plan.validate(json.dumps(f))
    assert plan.fused(json.dumps(f)) == f
    ops = by_name(f)
    # (join, the operator that receives its filters: the join, or its chain)
    joins = [(o, o["name"]) for o in f["ops"] if o["type"] == "HashJoinArrowPOp"]
    joins += [(j, o["name"]) for o in f["ops"] if o["type"] == "HashJoinChainPOp" for j in o["joins"]]
    for j, receiver in joins:
        for bf in j.get("buildFilters", []):
            # only inner joins on one key test filters, all on that key
            assert j.get("joinType", "INNER") == "INNER"
            assert bf["column"] == j["buildKey"]
            # the filter's creator (possibly merged into another operator) sends it to this join
            owner = next(o for o in f["ops"] if o["type"] == "BloomFilterCreatePOp" and
                         (o["name"] == bf["creator"] or
                          any(x.get("origin") == bf["creator"] for x in o.get("filters", []))))
            entries = owner.get("filters") or [dict(owner, origin=owner["name"])]
            entry = next(x for x in entries if x.get("origin", owner["name"]) == bf["creator"])
            assert receiver in entry["bloomFilterUsePOps"]
    # every bloom use left still has a filter for each of its columns
    for u in (o for o in f["ops"] if o["type"] == "BloomFilterUsePOp"):
        n = len(u.get("bloomFilterColumns", [u.get("bloomFilterColumn")]))
        assert len(u.get("creators", [None] * n)) == n
    assert ops["collate"]["type"] == "CollatePOp"


def test_fused_plan_text_round_trips_awkward_names():
    """Operator and column names with quotes, backslashes, control
    characters and non-ASCII bytes come back from gfpdb_plan_fuse as they
    went in."""
    names = ['q"uote', "back\\slash", "tab\there", "line\nbreak", "café ☃"]
    p = plan.Plan()
    prev = p.scan(names[0], "t", ["k"])
    for n in names[1:]:
        prev = p.filter(n, prev, None)
    p.collate("collate", prev)
    f = plan.fused(p)
    assert [o["name"] for o in f["ops"]] == names + ["collate"]
    assert f == plan.fused(json.dumps(f))


def test_plan_fuse_errors():
    import ctypes

    from flexpushdowndb_gb300 import _abi

    L = _abi.lib()
    need = ctypes.c_int64()
    assert L.gfpdb_plan_fuse(b"{not json", None, 0, ctypes.byref(need)) != 0
    assert "JSON" in L.gfpdb_last_error().decode()
    text = workloads.star_plan().to_json().encode()
    rc = L.gfpdb_plan_fuse(text, None, 0, ctypes.byref(need))
    assert rc != 0 and need.value > 1
    small = ctypes.create_string_buffer(need.value - 1)
    assert L.gfpdb_plan_fuse(text, small, need.value - 1, ctypes.byref(need)) != 0
    buf = ctypes.create_string_buffer(need.value)
    assert L.gfpdb_plan_fuse(text, buf, need.value, ctypes.byref(need)) == 0
    assert json.loads(buf.value.decode()) == plan.fused(workloads.star_plan())
    assert L.gfpdb_plan_fuse(None, None, 0, ctypes.byref(need)) != 0


def test_build_filter_not_folded_beside_another_build_producer():
    """A join whose build side has a second producer keeps its bloom use:
    the second producer's rows were never filtered."""
    p = plan.Plan()
    p.scan("scan_d", "dim", ["d_pk", "d_v"])
    p.scan("scan_e", "dim2", ["d_pk", "d_v"])
    p.scan("scan_f", "fact", ["fk", "x"])
    c = p.bloom_create("bw_create", "scan_f", "fk")
    u = p.bloom_use("bw_use", "scan_d", c, "d_pk")
    p.hash_join("join", u, c, "d_pk", "fk", ["x", "d_v"])
    p.op("join")["buildProducers"].append("scan_e")
    p.connect("scan_e", "join")
    p.collate("collate", "join")
    ops = by_name(plan.fused(p))
    assert "bw_use" in ops and "buildFilters" not in ops["join"]


def test_deeply_nested_plan_text_is_refused():
    """The plan reader descends recursively: nesting past 512 levels is an
    error, not a host stack overflow."""
    from flexpushdowndb_gb300 import _abi

    for text in ("[" * 200_000, '{"a":' * 200_000, '{"ops": ' + "[" * 600 + "]" * 600 + "}"):
        assert _abi.lib().gfpdb_plan_validate(text.encode()) != 0
        assert "nesting" in _abi.lib().gfpdb_last_error().decode()
    ok = '{"ops": ' + "[" * 100 + "]" * 100 + "}"
    _abi.lib().gfpdb_plan_validate(ok.encode())  # parses (and is refused only as a plan)
    assert "nesting" not in _abi.lib().gfpdb_last_error().decode()


def test_mutated_plans_validate_or_are_refused():
    """Random edits of plan texts (bytes changed, dropped, inserted;
    truncations): the plan checker and the fusion passes return a status,
    never crash."""
    import ctypes
    import random

    from flexpushdowndb_gb300 import _abi

    L = _abi.lib()
    base = [workloads.star_plan().to_json(), workloads.star_plan_planned().to_json(),
            workloads.two_table_plan().to_json()]
    rng = random.Random(77)
    alphabet = b'{}[]",:0123456789-.eE truefalsnul\\/abcdXYZ\xff'
    need = ctypes.c_int64()
    valid = 0
    for _ in range(1500):
        b = bytearray(rng.choice(base).encode())
        for _ in range(rng.randint(1, 6)):
            r, i = rng.random(), rng.randrange(len(b))
            if r < 0.5:
                b[i] = rng.choice(alphabet)
            elif r < 0.75:
                del b[i]
            else:
                b.insert(i, rng.choice(alphabet))
        if rng.random() < 0.05:
            b = b[:rng.randrange(len(b))]
        valid += L.gfpdb_plan_validate(bytes(b)) == 0
        L.gfpdb_plan_fuse(bytes(b), None, 0, ctypes.byref(need))
    assert 0 < valid < 1500
