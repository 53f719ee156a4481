"""Batched star queries (gfpdb_star_batch): every query of a batch must equal
its own single-query result, bit-exact, across uneven fact partitions."""

import numpy as np
import pytest

from flexpushdowndb_gb300 import GfpdbError, batch, plan, workloads
from flexpushdowndb_gb300.tupleset import Column, DeviceTable, Table
from oracle import queries

pytestmark = pytest.mark.gpu


def small_batch(n_parts=6, n_queries=8, seed=4000):
    sizes = workloads.batch_partition_sizes(n_parts, lo=1_000, hi=120_000, seed=seed)
    tabs = workloads.batch_tables(n_parts, sizes=sizes, seed=seed)
    qs = workloads.batch_queries(n_queries, seed=seed + 1)
    return tabs, [f"p{i}" for i in range(n_parts)], qs


def device(tabs):
    return plan.PreparedInputs({k: DeviceTable.from_host(v) for k, v in tabs.items()})


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_oracle_per_query(gpu, use_graph):
    tabs, parts, qs = small_batch()
    dev = device(tabs)
    spec = workloads.star_batch_spec(parts, qs)
    for _ in range(3):  # with a graph: capture, then replays
        got = batch.split_by_query(batch.star_batch(spec, dev, use_graph=use_graph).table)
        for q, ranges in enumerate(qs):
            want = queries.star_query_ranges(tabs, parts, ranges).sorted_rows()
            assert got.get(q, []) == want, f"query {q}"


def test_batch_equals_single_query_plans(gpu):
    tabs, parts, qs = small_batch(n_parts=4, n_queries=5, seed=4010)
    dev = device(tabs)
    got = batch.split_by_query(batch.star_batch(workloads.star_batch_spec(parts, qs), dev).table)
    for q, ranges in enumerate(qs):
        single = plan.execute(workloads.star_plan(ranges=ranges, fact_tables=parts), dev).table
        assert got.get(q, []) == single.sorted_rows(), f"query {q}"


@pytest.mark.parametrize("items,blocks,lf,order", [(1, 1, 0.25, (0, 1, 2, 3)), (8, 8, 0.9, (3, 2, 1, 0)),
                                                   (16, 2, 0.5, (1, 2, 3, 0))])
def test_batch_tuning_knobs_keep_results(gpu, items, blocks, lf, order):
    tabs, parts, qs = small_batch(n_parts=3, n_queries=6, seed=4020)
    dev = device(tabs)
    spec = workloads.star_batch_spec(parts, qs, load_factor=lf, items_per_thread=items, blocks_per_sm=blocks,
                                     probe_order=order)
    got = batch.split_by_query(batch.star_batch(spec, dev).table)
    for q, ranges in enumerate(qs):
        assert got.get(q, []) == queries.star_query_ranges(tabs, parts, ranges).sorted_rows()


def test_batch_empty_and_full_ranges(gpu):
    tabs, parts, _ = small_batch(n_parts=2, seed=4030)
    qs = [[(5, 4)] * 4, [(0, 99)] * 4, [(0, 0), (0, 99), (0, 99), (0, 99)]]  # empty, everything, one value
    got = batch.split_by_query(batch.star_batch(workloads.star_batch_spec(parts, qs), device(tabs)).table)
    assert 0 not in got
    for q in (1, 2):
        assert got[q] == queries.star_query_ranges(tabs, parts, qs[q]).sorted_rows()


def test_batch_rejects_repeated_dimension_keys(gpu):
    tabs, parts, qs = small_batch(n_parts=2, n_queries=2, seed=4040)
    d = tabs["d3"]
    tabs["d3"] = Table([Column(c.name, c.type, np.concatenate([c.values, c.values[:5]])) for c in d.columns])
    with pytest.raises(GfpdbError) as ei:
        batch.star_batch(workloads.star_batch_spec(parts, qs), device(tabs))
    assert "repeats a key" in ei.value.message
