"""Whole queries through the C++ operators (gfpdb_execute_plan) on the GPU,
bit-exact against the oracle: the two-table query and the star query with
forward + backward bloom predicate transfer, from host and device inputs,
whole and chunked into many TupleSets."""

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
