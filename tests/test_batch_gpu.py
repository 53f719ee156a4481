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
                                                   (2, 2, 0.5, (1, 2, 3, 0)), (4, 3, 0.5, None)])
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


def _rekey(tabs, parts, scale, offset, dtype):
    """Dimension keys k -> k * scale + offset (and the foreign keys with
    them): sparse key ranges take the hash-table lookup path."""
    out = dict(tabs)
    for i in range(1, 5):
        d = tabs[f"d{i}"]
        out[f"d{i}"] = Table([Column(c.name, dtype if c.name.endswith("_pk") else c.type,
                                     c.values.astype(np.int64) * scale + offset if c.name.endswith("_pk") else c.values)
                              for c in d.columns])
    for p in parts:
        t = tabs[p]
        out[p] = Table([Column(c.name, dtype if c.name.startswith("fk") else c.type,
                               c.values.astype(np.int64) * scale + offset if c.name.startswith("fk") else c.values)
                        for c in t.columns])
    return out


@pytest.mark.parametrize("scale,offset,dtype", [(7919, -5_000_000, "int32"), (1 << 33, -(1 << 40), "int64"),
                                                (1, -(1 << 31) + 10, "int32")])
def test_batch_sparse_and_negative_keys(gpu, scale, offset, dtype):
    tabs, parts, qs = small_batch(n_parts=3, n_queries=6, seed=4050)
    tabs = _rekey(tabs, parts, scale, offset, dtype)
    got = batch.split_by_query(batch.star_batch(workloads.star_batch_spec(parts, qs), device(tabs)).table)
    for q, ranges in enumerate(qs):
        assert got.get(q, []) == queries.star_query_ranges(tabs, parts, ranges).sorted_rows(), f"query {q}"


@pytest.mark.parametrize("order", [(0, 1, 2), (0, 1, 2, 2), (0, 1, 2, 4)])
def test_batch_rejects_bad_probe_order(gpu, order):
    tabs, parts, qs = small_batch(n_parts=2, n_queries=2, seed=4060)
    with pytest.raises(GfpdbError) as ei:
        batch.star_batch(workloads.star_batch_spec(parts, qs, probe_order=order), device(tabs))
    assert "probeOrder" in ei.value.message


def test_batch_rejects_bad_items_per_thread(gpu):
    tabs, parts, qs = small_batch(n_parts=2, n_queries=2, seed=4070)
    with pytest.raises(GfpdbError) as ei:
        batch.star_batch(workloads.star_batch_spec(parts, qs, items_per_thread=16), device(tabs))
    assert "itemsPerThread" in ei.value.message


def test_batch_tiny_and_empty_partitions(gpu):
    """Partitions shorter than one 16-byte copy, empty ones, and tails that
    are not a multiple of 4 rows."""
    sizes = [0, 1, 3, 5, 0, 2049, 70_001, 2]
    tabs = workloads.batch_tables(len(sizes), sizes=sizes, seed=4080)
    parts = [f"p{i}" for i in range(len(sizes))]
    qs = workloads.batch_queries(5, seed=4081) + [[(0, 99)] * 4]
    for items in (1, 8):
        spec = workloads.star_batch_spec(parts, qs, items_per_thread=items)
        got = batch.split_by_query(batch.star_batch(spec, device(tabs)).table)
        for q, ranges in enumerate(qs):
            assert got.get(q, []) == queries.star_query_ranges(tabs, parts, ranges).sorted_rows(), f"query {q}"


def test_batch_unaligned_columns(gpu):
    """Foreign-key columns that do not start on a 16-byte boundary are read
    with plain loads instead of bulk copies; results are the same."""
    import torch

    tabs, parts, qs = small_batch(n_parts=3, n_queries=4, seed=4090)
    dev = {k: DeviceTable.from_host(v) for k, v in tabs.items()}
    for p in parts:
        dt = dev[p]
        shifted = []
        for ts in dt.tensors:
            views = []
            for t in ts:
                buf = torch.empty(t.numel() + 1, dtype=t.dtype, device=t.device)
                buf[1:] = t
                views.append(buf[1:])
            shifted.append(views)
        dev[p] = DeviceTable(dt.names, dt.types, shifted, dt.num_rows)
    got = batch.split_by_query(batch.star_batch(workloads.star_batch_spec(parts, qs), plan.PreparedInputs(dev)).table)
    for q, ranges in enumerate(qs):
        assert got.get(q, []) == queries.star_query_ranges(tabs, parts, ranges).sorted_rows(), f"query {q}"


@pytest.mark.parametrize("pinned,use_graph", [(True, True), (True, False), (False, True)])
def test_batch_host_inputs_are_copied_every_run(gpu, pinned, use_graph):
    """Host-resident tables: every run copies the columns the batch reads
    (dimensions, then the fact partitions in groups, each group's fact pass
    after its copies), so a change to the host buffers between runs shows up
    in the next result; the copied bytes are counted."""
    from flexpushdowndb_gb300.tupleset import export_host

    tabs, parts, qs = small_batch(n_parts=11, n_queries=7, seed=4050)
    exported = {k: export_host(v, pinned=pinned) for k, v in tabs.items()}
    inputs = plan.PreparedInputs(exported)
    spec = workloads.star_batch_spec(parts, qs)
    dev = batch.split_by_query(batch.star_batch(spec, device(tabs)).table)
    for _ in range(3):
        r = batch.star_batch(spec, inputs, use_graph=use_graph)
        assert batch.split_by_query(r.table) == dev
    # the batch reads fk1..fk4, qty, price_cents, discount and each dimension's key, filter and group column:
    # from pageable memory all of them are copied; from page-locked memory the columns read for some rows
    # only are read in place (declared as one 32-byte sector per row and column)
    fact_bytes = sum(tabs[p].num_rows * 32 for p in parts)
    dim_bytes = sum(tabs[f"d{i}"].num_rows * 4 * (3 if i in (2, 4) else 2) for i in range(1, 5))
    if pinned:
        assert dim_bytes < r.stats["h2d_bytes"]
    else:
        assert r.stats["h2d_bytes"] == fact_bytes + dim_bytes
    # change one partition's quantities and one dimension's filter column in the host buffers
    changed = dict(tabs)
    p3, d2 = tabs["p3"], tabs["d2"]
    new_qty = (p3["qty"] * 3 + 1).astype(np.int32)
    new_f = ((d2["d2_f"] + 17) % 100).astype(np.int32)
    changed["p3"] = Table([Column(c.name, c.type, new_qty if c.name == "qty" else c.values) for c in p3.columns])
    changed["d2"] = Table([Column(c.name, c.type, new_f if c.name == "d2_f" else c.values) for c in d2.columns])
    _overwrite_host(exported["p3"], "qty", new_qty)
    _overwrite_host(exported["d2"], "d2_f", new_f)
    got = batch.split_by_query(batch.star_batch(spec, inputs, use_graph=use_graph).table)
    for q, ranges in enumerate(qs):
        assert got.get(q, []) == queries.star_query_ranges(changed, parts, ranges).sorted_rows(), f"query {q}"


def _overwrite_host(ex, column, values):
    """Write new values into an exported host table's column buffer."""
    import ctypes

    names = [ex.schema.children[i].contents.name.decode() for i in range(ex.schema.n_children)]
    child = ex.array.array.children[names.index(column)].contents
    ctypes.memmove(child.buffers[1], np.ascontiguousarray(values).ctypes.data, values.nbytes)


@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("items,blocks", [(1, 1), (2, 2), (8, 3)])
def test_batch_direct_and_pipelined_fact_passes(gpu, direct, items, blocks):
    """The two forms of the fact pass (warps reading their own rows, or a
    copy pipeline feeding consumer warps) give every query its oracle rows,
    with partitions whose sizes leave ragged slices and tiles."""
    tabs, parts, qs = small_batch(n_parts=5, n_queries=33, seed=4060)  # 33 queries: 64-bit masks
    dev = device(tabs)
    for nq in (33, 9):  # and 32-bit masks
        spec = dict(workloads.star_batch_spec(parts, qs[:nq], items_per_thread=items, blocks_per_sm=blocks),
                    direct=direct)
        got = batch.split_by_query(batch.star_batch(spec, dev).table)
        for q in range(nq):
            assert got.get(q, []) == queries.star_query_ranges(tabs, parts, qs[q]).sorted_rows(), f"query {q}"


def test_prepared_batch_launch_wait(gpu):
    """Prepared batches (gfpdb_batch_prepare / launch / wait): results equal
    the one-call form's; two prepared copies run back to back; a second
    launch before the wait is refused, and so is a wait with nothing
    launched."""
    tabs, parts, qs = small_batch(n_parts=7, n_queries=12, seed=4070)
    dev = device(tabs)
    spec = workloads.star_batch_spec(parts, qs)
    want = batch.split_by_query(batch.star_batch(spec, dev).table)
    a, b = batch.PreparedBatch(spec, dev), batch.PreparedBatch(spec, dev)
    for _ in range(2):
        assert batch.split_by_query(a.execute().table) == want
    a.launch()
    for k in range(5):
        (b if k % 2 == 0 else a).launch()
        r = (a if k % 2 == 0 else b).wait()
        assert batch.split_by_query(r.table) == want
    assert batch.split_by_query(b.wait().table) == want
    b.launch()
    with pytest.raises(GfpdbError):
        b.launch()
    b.wait()
    with pytest.raises(GfpdbError):
        b.wait()
    # host inputs (pinned): re-read by every run
    from flexpushdowndb_gb300.tupleset import export_host

    exported = {k: export_host(v, pinned=True) for k, v in tabs.items()}
    h = batch.PreparedBatch(spec, plan.PreparedInputs(exported))
    r = h.execute()
    assert batch.split_by_query(r.table) == want
    assert r.stats["h2d_bytes"] > 0
    new_qty = (tabs["p2"]["qty"] + 5).astype(np.int32)
    _overwrite_host(exported["p2"], "qty", new_qty)
    changed = dict(tabs)
    changed["p2"] = Table([Column(c.name, c.type, new_qty if c.name == "qty" else c.values) for c in tabs["p2"].columns])
    got = batch.split_by_query(h.execute().table)
    for q, ranges in enumerate(qs):
        assert got.get(q, []) == queries.star_query_ranges(changed, parts, ranges).sorted_rows(), f"query {q}"
