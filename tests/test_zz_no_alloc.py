"""gfpdb_filter_evaluate_noalloc: the filter for callers that cannot allocate
device memory (graph capture, fixed device arenas, foreign allocators).

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
                  Column("d", "date32", rng.integers(8000, 11000, n))])


def noalloc(filt, dev_table, project, stream=None):
    """Call the entry point with caller-allocated (torch) output buffers."""
    import torch

    ex = dev_table.export()
    outs = []
    for name in project:
        ty = dev_table.types[dev_table.names.index(name)]
        outs.append(torch.empty(dev_table.num_rows if dev_table.num_rows else 1,
                                dtype=torch.int64 if ty == "int64" else torch.int32, device="cuda"))
    ptrs = (ctypes.c_void_p * len(outs))(*[t.data_ptr() for t in outs])
    n_out = ctypes.c_int64(-1)
    rc = _abi.lib().gfpdb_filter_evaluate_noalloc(filt._h, ex.schema_ptr, ex.array_ptr, _abi.cstr_array(project),
                                                   len(project), ptrs, ctypes.byref(n_out), stream)
    _abi.check(rc)
    return [t[: n_out.value].cpu().numpy() for t in outs], n_out.value


@pytest.mark.parametrize("n", [100_003, 4096])
def test_noalloc_matches_filter_evaluate_twice(n):
    ops.init(0)
    t = make_table(n, seed=n)
    dev = DeviceTable.from_host(t)
    project = ["b", "a", "d"]
    preds = [and_(gt(col("a"), num_lit(-100)), lt(col("b"), num_lit(0, "int64"))),
             lt(col("d"), num_lit(9000, "date32"))]
    for pred in preds:
        filt = ops.Filter(pred, t)
        want = filt.evaluate(dev, project=project)
        for _ in range(2):  # two calls in a row reuse the same scratch
            got, n_out = noalloc(filt, dev, project)
            assert n_out == want.num_rows
            for name, arr in zip(project, got):
                assert np.array_equal(arr, want[name]), name


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
