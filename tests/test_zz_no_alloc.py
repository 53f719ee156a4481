"""gfpdb_filter_evaluate_noalloc: the filter for callers that cannot allocate
device memory (engines that budget a fixed device arena themselves, and
embedders whose device memory belongs to another runtime's allocator).

It must select exactly what gfpdb_filter_evaluate selects while allocating
nothing itself: its scratch is a file-scope device array and the caller owns
the output buffers. Two calls in a row check that each call clears the
shared scratch it reuses. This file sorts last so that a run stopping at the
first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest

from flexpushdowndb_gb300 import _abi, ops
from flexpushdowndb_gb300.expression import and_, col, gt, lt, num_lit
from flexpushdowndb_gb300.tupleset import Column, DeviceTable, Table

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 28


def make_table(n, seed):
    rng = np.random.default_rng(seed)
    return Table([Column("a", "int32", rng.integers(-500, 500, n)),
                  Column("b", "int64", rng.integers(-10**12, 10**12, n)),
                  Column("d", "date32", rng.integers(8000, 11000, n)),
                  Column("s", "utf8", [f"v{i % 7}" for i in range(n)])])


def call_noalloc(filt, ex, types, rows, project, stream=None):
    """Call the entry point on an export with caller-allocated (torch)
    output buffers; returns (status, selected columns, selected rows)."""
    import torch

    outs = [torch.empty(max(1, rows), dtype=torch.int64 if types[name] == "int64" else torch.int32, device="cuda")
            for name in project]
    ptrs = (ctypes.c_void_p * max(1, len(outs)))(*[t.data_ptr() for t in outs])
    n_out = ctypes.c_int64(-1)
    rc = _abi.lib().gfpdb_filter_evaluate_noalloc(filt._h, ex.schema_ptr, ex.array_ptr, _abi.cstr_array(project),
                                                   len(project), ptrs, ctypes.byref(n_out), stream)
    if rc != _abi.GFPDB_OK:
        return rc, None, None
    return rc, [t[: n_out.value].cpu().numpy() for t in outs], n_out.value


def noalloc(filt, dev_table, project):
    types = dict(zip(dev_table.names, dev_table.types))
    ex = dev_table.export()
    rc, got, n = call_noalloc(filt, ex, types, dev_table.num_rows, project)
    _abi.check(rc)
    return got, n


PREDS = [and_(gt(col("a"), num_lit(-100)), lt(col("b"), num_lit(0, "int64"))),
         lt(col("d"), num_lit(9000, "date32"))]


@pytest.mark.parametrize("n", [100_003, 4096])
def test_noalloc_matches_filter_evaluate_twice(n):
    ops.init(0)
    t = make_table(n, seed=n)
    dev = DeviceTable.from_host(t)
    project = ["b", "a", "d"]
    for pred in PREDS:
        filt = ops.Filter(pred, t)
        want = filt.evaluate(dev, project=project)
        for _ in range(2):  # two calls in a row reuse the same scratch
            got, n_out = noalloc(filt, dev, project)
            assert n_out == want.num_rows
            for name, arr in zip(project, got):
                assert np.array_equal(arr, want[name]), name


def test_noalloc_allocates_nothing():
    ops.init(0)
    t = make_table(50_000, seed=5)
    dev = DeviceTable.from_host(t)
    filt = ops.Filter(PREDS[0], t)
    L = _abi.lib()
    noalloc(filt, dev, ["a"])  # the first call on the device looks up the scratch address
    before = L.gfpdb_thread_device_alloc_bytes()
    noalloc(filt, dev, ["a", "b"])
    assert L.gfpdb_thread_device_alloc_bytes() == before
    filt.evaluate(dev, project=["a"])  # the allocating entry point moves the counter
    assert L.gfpdb_thread_device_alloc_bytes() > before


def test_noalloc_sliced_input():
    """A struct offset (odd, so the columns are not 16-byte aligned) and a
    child offset of its own: the call reads the same rows as an unsliced
    table holding them."""
    ops.init(0)
    n, soff = 70_001, 3
    t = make_table(n, seed=9)
    dev = DeviceTable.from_host(t)
    ex = dev.export()
    ex.array.array.offset = soff
    ex.array.array.length = n - soff - 1
    b = ex.array.array.children[dev.names.index("b")].contents
    b.offset = 1  # column b's logical row k is its buffer's row k + 1
    b.length = n - 1
    sliced = Table([Column("a", "int32", t["a"][soff:n - 1]), Column("b", "int64", t["b"][soff + 1:n]),
                    Column("d", "date32", t["d"][soff:n - 1])])
    project = ["a", "b", "d"]
    types = dict(zip(dev.names, dev.types))
    for pred in PREDS:
        filt = ops.Filter(pred, t)
        want = filt.evaluate(DeviceTable.from_host(sliced), project=project)
        for _ in range(2):
            rc, got, n_out = call_noalloc(filt, ex, types, n, project)
            assert rc == _abi.GFPDB_OK, _abi.lib().gfpdb_last_error()
            assert n_out == want.num_rows
            for name, arr in zip(project, got):
                assert np.array_equal(arr, want[name]), name


def test_noalloc_rejects_bad_inputs():
    ops.init(0)
    L = _abi.lib()
    t = make_table(1000, seed=2)
    dev = DeviceTable.from_host(t)
    types = dict(zip(dev.names, dev.types))
    filt = ops.Filter(gt(col("a"), num_lit(0)), t)
    # utf8 outputs need an allocation
    rc, _, _ = call_noalloc(filt, dev.export(), types, 1000, ["s"])
    assert rc == _abi.GFPDB_EUNSUPPORTED
    # a child shorter than the struct
    ex = dev.export()
    ex.array.array.children[dev.names.index("a")].contents.length = 999
    rc, _, _ = call_noalloc(filt, ex, types, 1000, ["b"])
    assert rc == _abi.GFPDB_EINVAL and b"shorter" in L.gfpdb_last_error()
    # a nullable predicate column and a nullable output column
    for name, project in (("a", ["b"]), ("d", ["d"])):
        ex = dev.export()
        child = ex.array.array.children[dev.names.index(name)].contents
        validity = (ctypes.c_uint8 * 128)()
        child.null_count = 1
        child.buffers[0] = ctypes.addressof(validity)
        rc, _, _ = call_noalloc(filt, ex, types, 1000, project)
        assert rc == _abi.GFPDB_EUNSUPPORTED and b"nulls" in L.gfpdb_last_error()
    # struct-level nulls
    ex = dev.export()
    ex.array.array.null_count = 1
    rc, _, _ = call_noalloc(filt, ex, types, 1000, ["b"])
    assert rc == _abi.GFPDB_EUNSUPPORTED
    # the device still answers
    got, n_out = noalloc(filt, dev, ["a"])
    assert n_out == int(np.sum(t["a"] > 0))


def test_noalloc_rejects_oversized_input():
    ops.init(0)
    t = make_table(16, seed=1)
    dev = DeviceTable.from_host(t)
    filt = ops.Filter(gt(col("a"), num_lit(0)), t)
    ex = dev.export()
    ex.array.array.length = MAX_ROWS + 1  # rejected before any device access
    ptrs = (ctypes.c_void_p * 1)(None)
    n_out = ctypes.c_int64(0)
    rc = _abi.lib().gfpdb_filter_evaluate_noalloc(filt._h, ex.schema_ptr, ex.array_ptr, _abi.cstr_array(["a"]), 1,
                                                   ptrs, ctypes.byref(n_out), None)
    assert rc == _abi.GFPDB_EINVAL
    assert b"maximum" in _abi.lib().gfpdb_last_error()
