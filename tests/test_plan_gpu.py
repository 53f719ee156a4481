"""Whole queries through the C++ operators (gfpdb_execute_plan) on the GPU,
bit-exact against the oracle: the two-table query and the star query with
forward + backward bloom predicate transfer, from host and device inputs,
whole and chunked into many TupleSets."""

import json

import pytest

from flexpushdowndb_gb300 import GfpdbError, plan, workloads
from flexpushdowndb_gb300.tupleset import DeviceTable
from oracle import queries

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fact_rows,chunk", [(0, 0), (1, 0), (50_000, 0), (1_000_000, 0), (1_000_000, 100_000)])
def test_two_table_query(gpu, fact_rows, chunk):
    tabs = workloads.two_table_tables(fact_rows=fact_rows)
    got = plan.execute(workloads.two_table_plan(chunk_rows=chunk), tabs)
    want = queries.two_table_query(tabs)
    assert got.table.names == ["region", "revenue", "cnt"]
    assert got.table.sorted_rows() == want.sorted_rows()
    assert got.stats["kernel_launches"] > 0


@pytest.mark.parametrize("fact_rows,chunk,device", [(100_000, 0, False), (600_000, 150_000, True),
                                                    (6_000_000, 0, True)])
def test_star_query(gpu, fact_rows, chunk, device):
    tabs = workloads.star_tables(fact_rows=fact_rows)
    inputs = {k: DeviceTable.from_host(v) for k, v in tabs.items()} if device else tabs
    got = plan.execute(workloads.star_plan(chunk_rows=chunk), inputs)
    want = queries.star_query(tabs)
    assert got.table.names == ["d2_g", "d4_g", "revenue", "discount_revenue", "cnt"]
    assert got.table.sorted_rows() == want.sorted_rows()
    # blooms only remove rows that cannot join
    assert want.sorted_rows() == queries.star_query_direct(tabs).sorted_rows()


@pytest.mark.parametrize("consts", [(0, 0, 0, 0), (4, 24, 6, 6), (2, 11, 3, 1)])
def test_star_query_variants(gpu, consts):
    tabs = workloads.star_tables(fact_rows=400_000, seed=2000 + sum(consts))
    got = plan.execute(workloads.star_plan(consts=consts), tabs)
    assert got.table.sorted_rows() == queries.star_query(tabs, consts=consts).sorted_rows()


def test_star_query_forward_only(gpu):
    tabs = workloads.star_tables(fact_rows=200_000)
    got = plan.execute(workloads.star_plan(backward=False), tabs)
    assert got.table.sorted_rows() == queries.star_query_direct(tabs).sorted_rows()


@pytest.mark.parametrize("deferred", [True, False])
def test_star_query_deferred_and_exact_sizes(gpu, deferred):
    tabs = workloads.star_tables(fact_rows=300_000, seed=2024)
    p = workloads.star_plan()
    text = p.to_json()[:-1] + f',"deferredSizes":{"true" if deferred else "false"}}}'
    got = plan.execute(text, tabs)
    assert got.table.sorted_rows() == queries.star_query(tabs).sorted_rows()


def _with_options(p, **opts):
    import json

    d = json.loads(p.to_json())
    d.update(opts)
    return json.dumps(d)


def test_star_query_cuda_graph_capture_and_replay(gpu):
    tabs = workloads.star_tables(fact_rows=500_000, seed=77)
    dev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
    text = _with_options(workloads.star_plan(), cudaGraph=True)
    want = queries.star_query(tabs).sorted_rows()
    for _ in range(4):  # capture on the first call, replays after
        got = plan.execute(text, dev)
        assert got.table.sorted_rows() == want
    # other input buffers: a new capture for them
    tabs2 = workloads.star_tables(fact_rows=500_000, seed=78)
    dev2 = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs2.items()})
    for _ in range(2):
        assert plan.execute(text, dev2).table.sorted_rows() == queries.star_query(tabs2).sorted_rows()
    # the first inputs' graph is still valid
    assert plan.execute(text, dev).table.sorted_rows() == want


def test_cuda_graph_with_host_inputs_and_fallback(gpu):
    # pinned host inputs: the host-to-device copies are part of the graph
    tabs = workloads.star_tables(fact_rows=200_000, seed=5)
    pinned = plan.PreparedInputs(tabs, pinned=True)
    text = _with_options(workloads.star_plan(), cudaGraph=True)
    want = queries.star_query(tabs).sorted_rows()
    for _ in range(3):
        assert plan.execute(text, pinned).table.sorted_rows() == want
    # a utf8 group key needs the host mid-plan: capture is refused and every
    # call runs the ordinary path
    t2 = workloads.two_table_tables(fact_rows=100_000)
    text2 = _with_options(workloads.two_table_plan(), cudaGraph=True)
    for _ in range(3):
        assert plan.execute(text2, t2).table.sorted_rows() == queries.two_table_query(t2).sorted_rows()


@pytest.mark.parametrize("mode", ["engine", "sm", "zerocopy"])
@pytest.mark.parametrize("graph", [False, True])
def test_host_input_copy_modes(gpu, mode, graph):
    tabs = workloads.star_tables(fact_rows=300_000, seed=31)
    pinned = plan.PreparedInputs(tabs, pinned=True)
    text = _with_options(workloads.star_plan(), hostCopy=mode, cudaGraph=graph)
    want = queries.star_query(tabs).sorted_rows()
    for _ in range(3 if graph else 1):
        assert plan.execute(text, pinned).table.sorted_rows() == want


@pytest.mark.parametrize("fuse", [True, False])
def test_bloom_chain_fusion_same_result(gpu, fuse):
    tabs = workloads.star_tables(fact_rows=400_000, seed=99)
    r = plan.execute(_with_options(workloads.star_plan(), fusePipelines=fuse), tabs)
    assert r.table.sorted_rows() == queries.star_query(tabs).sorted_rows()
    # the four forward BloomFilterUsePOps on the fact table fuse into one,
    # the four backward ones fold into the join builds, their four creators
    # into one, the four joins into one chain
    assert r.stats["num_ops"] == (18 if fuse else 31)


def test_duplicate_build_keys_rerun_with_exact_sizes(gpu):
    # Every dim key appears twice, so each matching fact row joins two dim
    # rows and the join output exceeds the probe side's row count: the
    # deferred run overflows and the plan is re-run with exact sizes.
    import numpy as np

    from flexpushdowndb_gb300.tupleset import Column, Table
    from oracle import ops as oops

    tabs = workloads.two_table_tables(fact_rows=50_000, dim_rows=2_000)
    d = tabs["dim"]
    dup = Table([Column(c.name, c.type, np.concatenate([c.values, c.values]) if c.type != "utf8" else
                        d[c.name] + d[c.name]) for c in d.columns])
    tabs2 = {"fact": tabs["fact"], "dim": dup}
    got = plan.execute(workloads.two_table_plan(), tabs2)
    want = queries.two_table_query(tabs2)
    assert got.table.sorted_rows() == want.sorted_rows()
    assert sum(r[-1] for r in want.rows()) > 0


def test_plan_errors_surface_as_error_messages(gpu):
    tabs = workloads.two_table_tables(fact_rows=1000)
    p = workloads.two_table_plan()
    p.op("join")["probeKey"] = "no_such_column"
    with pytest.raises(GfpdbError) as ei:
        plan.execute(p, tabs)
    assert "no_such_column" in ei.value.message and "join" in ei.value.message
    with pytest.raises(GfpdbError) as ei:
        plan.execute(workloads.two_table_plan(), {"fact": tabs["fact"]})
    assert "dim" in ei.value.message
    # the device is still usable after an operator error
    ok = plan.execute(workloads.two_table_plan(), tabs)
    assert ok.table.sorted_rows() == queries.two_table_query(tabs).sorted_rows()


@pytest.mark.parametrize("streams,graph,deferred", [(1, False, True), (4, False, True), (8, False, False),
                                                    (4, True, True), (16, True, True), (2, False, True)])
def test_streams_same_result(gpu, streams, graph, deferred):
    """Operators on independent plan branches run on their own streams (and
    as parallel graph branches); results equal the single-stream run's and
    the oracle's, for the star query and the chunked two-table query."""
    tabs = workloads.star_tables(fact_rows=1_500_000, seed=2300 + streams)
    dev = plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})
    text = _with_options(workloads.star_plan(), streams=streams, cudaGraph=graph, deferredSizes=deferred)
    want = queries.star_query(tabs).sorted_rows()
    for _ in range(3):  # with a graph: capture, then replays
        assert plan.execute(text, dev).table.sorted_rows() == want
    t2 = workloads.two_table_tables(fact_rows=700_000, seed=2400 + streams)
    text2 = _with_options(workloads.two_table_plan(chunk_rows=100_000), streams=streams, cudaGraph=graph)
    assert plan.execute(text2, t2).table.sorted_rows() == queries.two_table_query(t2).sorted_rows()


def test_streams_option_validated(gpu):
    with pytest.raises(GfpdbError):
        plan.execute(_with_options(workloads.star_plan(), streams=0), workloads.star_tables(fact_rows=1000))


def test_aggregate_pop_matches_oracle(gpu):
    """AggregatePOp: one row of non-grouped sums/counts/min/max; no rows in
    (every row filtered out) gives no rows out."""
    from flexpushdowndb_gb300.expression import col, lt, num_lit, times
    from flexpushdowndb_gb300.ops import aggregate
    from oracle import ops as oops

    tabs = workloads.two_table_tables(fact_rows=300_000, seed=2500)
    for cut in (25, 0):
        p = plan.Plan()
        p.scan("scan", "fact", ["fk", "qty", "price_cents"])
        p.filter("f", "scan", lt(col("qty"), num_lit(cut)))
        aggs = [aggregate("SUM", "rev", times(col("price_cents"), col("qty"))), aggregate("COUNT", "n"),
                aggregate("MIN", "lo", col("price_cents")), aggregate("MAX", "hi", col("fk"))]
        p.aggregate("agg", "f", aggs)
        p.collate("collate", "agg")
        got = plan.execute(p, tabs).table
        sel = oops.filter_table(tabs["fact"], lt(col("qty"), num_lit(cut)))
        if sel.num_rows == 0:
            assert got.num_rows == 0
            continue
        want = oops.group_by(sel, [], [{"function": "SUM", "name": "rev", "expr": times(col("price_cents"), col("qty"))},
                                        {"function": "COUNT", "name": "n"},
                                        {"function": "MIN", "name": "lo", "expr": col("price_cents")},
                                        {"function": "MAX", "name": "hi", "expr": col("fk")}])
        assert got.rows() == want.rows()


def _snowflake_tables(n_fact, seed, dup):
    """fact -> a (on fk_a) -> b (on a_link, a column of a's rows); a and b
    keys repeated `dup` times."""
    import numpy as np

    from flexpushdowndb_gb300.tupleset import Column, Table

    rng = np.random.default_rng(seed)
    na, nb = 3_000, 500
    a_keys = np.repeat(np.arange(na, dtype=np.int64), dup)
    b_keys = np.repeat(np.arange(nb, dtype=np.int64) * 7, dup)
    fact = Table([Column("fk_a", "int32", rng.integers(-10, na + 10, n_fact)),
                  Column("v", "int64", rng.integers(-10**12, 10**12, n_fact)),
                  Column("w", "int32", rng.integers(0, 100, n_fact))])
    a = Table([Column("a_pk", "int32", a_keys), Column("a_link", "int64", rng.integers(0, nb, len(a_keys)) * 7),
               Column("a_x", "int32", rng.integers(0, 1000, len(a_keys))),
               Column("a_s", "utf8", [f"s{int(x) % 17}" for x in a_keys])])
    b = Table([Column("b_pk", "int64", b_keys), Column("b_y", "int64", rng.integers(-50, 50, len(b_keys)))])
    return {"fact": fact, "a": a, "b": b}


def _snowflake_plan(project_utf8, fuse):
    p = plan.Plan()
    p.scan("scan_a", "a", ["a_pk", "a_link", "a_x", "a_s"])
    p.scan("scan_b", "b", ["b_pk", "b_y"])
    p.scan("scan_fact", "fact", ["fk_a", "v", "w"])
    p.hash_join("join_a", "scan_a", "scan_fact", "a_pk", "fk_a",
                ["v", "w", "a_link", "a_x"] + (["a_s"] if project_utf8 else []))
    p.hash_join("join_b", "scan_b", "join_a", "b_pk", "a_link", ["v", "a_x", "b_y", "w"] + (["a_s"] if project_utf8 else []))
    p.collate("collate", "join_b")
    d = json.loads(p.to_json())
    d["fusePipelines"] = fuse
    return json.dumps(d)


@pytest.mark.parametrize("dup", [1, 3])
@pytest.mark.parametrize("project_utf8", [False, True])
@pytest.mark.parametrize("graph", [False, True])
def test_join_chain_snowflake_duplicates(gpu, dup, project_utf8, graph):
    """A join chain whose second key comes from the first join's build rows
    (int64 key against an int64 build key), with repeated build keys (more
    output rows than input rows: the deferred run overflows and is re-run
    exactly) and with a utf8 output (the chain then runs join by join):
    fused and unfused plans match the oracle."""
    from oracle import ops as oops

    tabs = _snowflake_tables(40_000, 3000 + dup, dup)
    j1 = oops.hash_join(tabs["a"], tabs["fact"], "a_pk", "fk_a",
                        ["v", "w", "a_link", "a_x"] + (["a_s"] if project_utf8 else []))
    want = oops.hash_join(tabs["b"], j1, "b_pk", "a_link", ["v", "a_x", "b_y", "w"] + (["a_s"] if project_utf8 else []))
    for fuse in (True, False):
        text = _snowflake_plan(project_utf8, fuse)
        if graph:
            text = json.dumps(dict(json.loads(text), cudaGraph=True))
        for _ in range(2 if graph else 1):
            r = plan.execute(text, tabs)
            assert r.table.names == want.names
            assert r.table.sorted_rows() == want.sorted_rows()
        assert r.stats["num_ops"] == (5 if fuse else 6)


def test_join_chain_large_input_staged_output(gpu):
    """A chain over more than a million input rows stages its output rows
    per warp before writing them: same rows as the oracle, with repeated
    build keys so that a warp flushes many times."""
    from oracle import ops as oops

    tabs = _snowflake_tables(1_100_000, 4242, 2)
    j1 = oops.hash_join(tabs["a"], tabs["fact"], "a_pk", "fk_a", ["v", "w", "a_link", "a_x"])
    want = oops.hash_join(tabs["b"], j1, "b_pk", "a_link", ["v", "a_x", "b_y", "w"])
    r = plan.execute(_snowflake_plan(False, True), tabs)
    assert r.stats["num_ops"] == 5
    assert r.table.num_rows == want.num_rows
    assert r.table.sorted_rows() == want.sorted_rows()


@pytest.mark.parametrize("graph", [False, True])
def test_prepared_plan_matches_execute(gpu, graph):
    """PreparedPlan (bound inputs, one-call result import) returns what
    plan.execute returns, call after call, with host and device results of
    fixed-width and utf8 columns."""
    tabs = workloads.two_table_tables(fact_rows=200_000)
    text = _with_options(workloads.two_table_plan(), cudaGraph=graph)
    want = plan.execute(text, tabs).table
    pp = plan.PreparedPlan(text, plan.PreparedInputs(tabs))
    for _ in range(3):
        got = pp.execute().table
        assert got.names == want.names
        assert got.sorted_rows() == want.sorted_rows()

def test_prepared_plans_launched_back_to_back(gpu):
    """Two prepared plans of the star query (graph instances 0 and 1, so each
    has its own capture) launched alternately on one stream, each waited for
    while the other runs: every result, through the first runs, the captures
    and the replays, matches the oracle; a second launch before the wait and
    a wait without a launch are errors."""
    from flexpushdowndb_gb300 import _abi

    tabs = workloads.star_tables(fact_rows=300_000, seed=43)
    want = queries.star_query(tabs).sorted_rows()
    inputs = plan.PreparedInputs(tabs)
    base = json.loads(_with_options(workloads.star_plan(), cudaGraph=True))
    pps = [plan.PreparedPlan(json.dumps(dict(base, graphInstance=i)), inputs) for i in (0, 1)]
    pps[0].launch()
    for k in range(1, 9):
        pps[k % 2].launch()
        r = pps[(k - 1) % 2].wait()
        assert r.table.sorted_rows() == want
    r = pps[0].wait()
    assert r.table.sorted_rows() == want
    assert r.stats["device_ns"] > 0  # a replay
    # a replay's stats are its own, not the other instance's as well
    alone = plan.PreparedPlan(json.dumps(dict(base, graphInstance=2)), inputs)
    for _ in range(3):
        r_alone = alone.execute()
    for k in ("kernel_launches", "h2d_bytes", "d2h_bytes", "num_ops"):
        assert r.stats[k] == r_alone.stats[k], k
    pps[1].launch()
    with pytest.raises(_abi.GfpdbError):
        pps[1].launch()
    assert pps[1].wait().table.sorted_rows() == want
    with pytest.raises(_abi.GfpdbError):
        pps[1].wait()
    # the same text prepared twice shares one capture: while one copy's
    # replay is in flight the other's launch is refused, not overlapped
    twin = plan.PreparedPlan(json.dumps(dict(base, graphInstance=0)), inputs)
    pps[0].launch()
    with pytest.raises(_abi.GfpdbError) as ei:
        twin.launch()
    assert "graphInstance" in ei.value.message
    assert pps[0].wait().table.sorted_rows() == want
    assert twin.execute().table.sorted_rows() == want


def test_prepared_star_plan_through_capture_and_replays(gpu):
    """A prepared star plan: the first runs take the ordinary path (run,
    then capture), later ones replay the graph; every result matches the
    oracle and each call returns its own copy."""
    tabs = workloads.star_tables(fact_rows=500_000, seed=41)
    want = queries.star_query(tabs).sorted_rows()
    pp = plan.PreparedPlan(_with_options(workloads.star_plan(), cudaGraph=True), plan.PreparedInputs(tabs))
    results = [pp.execute() for _ in range(4)]
    for r in results:
        assert r.table.sorted_rows() == want
    assert results[-1].stats["device_ns"] > 0  # a replay


@pytest.mark.parametrize("graph", [False, True])
def test_star_plan_with_fact_columns_read_in_place(gpu, graph):
    """Pinned host inputs, the fact columns other than the first probe key
    read in place: the same result as device inputs; the declared host bytes
    count the in-place columns whole."""
    tabs = workloads.star_tables(fact_rows=500_000, seed=2024)
    d = json.loads(workloads.star_plan().to_json())
    for o in d["ops"]:
        if o["type"] == "TableScanPOp" and o["table"] == "fact":
            o["inPlaceColumns"] = [c for c in o["columns"] if c != "fk2"]
    d["cudaGraph"] = graph
    host = plan.PreparedInputs(tabs, pinned=True)
    want = queries.star_query(tabs).sorted_rows()
    for _ in range(3 if graph else 1):
        res = plan.execute(json.dumps(d), host)
        assert res.table.sorted_rows() == want
    fact_bytes = sum(c.values.nbytes for c in tabs["fact"].columns)
    assert res.stats["h2d_bytes"] >= fact_bytes
