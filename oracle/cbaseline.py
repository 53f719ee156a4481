"""ctypes wrapper of oracle/baseline.c (BENCHMARK / TEST INFRASTRUCTURE ONLY)."""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

from flexpushdowndb_gb300.tupleset import Column, Table

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"


class _Fact(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("fk", ctypes.c_void_p * 4), ("qty", ctypes.c_void_p),
                ("price", ctypes.c_void_p), ("disc", ctypes.c_void_p)]


class _Dim(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("pk", ctypes.c_void_p), ("f", ctypes.c_void_p), ("g", ctypes.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        _lib = ctypes.CDLL(str(LIB))
        _lib.orc_star_query.restype = ctypes.c_int64
        _lib.orc_star_query_parts.restype = ctypes.c_int64
    return _lib


class StarInputs:
    """Arrays of a star workload laid out for the C baseline (kept alive):
    the dimensions d1..d4 and the fact table, or the fact partitions named
    in `parts`."""

    def __init__(self, tables: dict[str, Table], parts=("fact",)):
        self.keep = []

        def arr(t: Table, name: str, dt):
            a = np.ascontiguousarray(t[name], dtype=dt)
            self.keep.append(a)
            return a.ctypes.data

        self.n_parts = len(parts)
        self.parts = (_Fact * len(parts))()
        for j, name in enumerate(parts):
            f = tables[name]
            fp = self.parts[j]
            fp.n = f.num_rows
            for i in range(4):
                fp.fk[i] = arr(f, f"fk{i + 1}", np.int32)
            fp.qty = arr(f, "qty", np.int32)
            fp.price = arr(f, "price_cents", np.int64)
            fp.disc = arr(f, "discount", np.int32)
        self.fact = self.parts[0]
        self.rows = sum(self.parts[j].n for j in range(len(parts)))
        self.dims = (_Dim * 4)()
        for i in range(4):
            d = tables[f"d{i + 1}"]
            self.dims[i].n = d.num_rows
            self.dims[i].pk = arr(d, f"d{i + 1}_pk", np.int32)
            self.dims[i].f = arr(d, f"d{i + 1}_f", np.int32)
            self.dims[i].g = arr(d, f"d{i + 1}_g", np.int32)


def star_query(inputs: StarInputs, consts=(1, 3, 2, 5), bits: int = 10, nh: int = 3, threads: int | None = None,
               max_groups: int = 4096) -> Table:
    """The star query with dimension filters f == consts[i]."""
    return star_query_ranges(inputs, [(c, c) for c in consts], bits, nh, threads, max_groups)


def star_query_ranges(inputs: StarInputs, ranges, bits: int = 10, nh: int = 3, threads: int | None = None,
                      max_groups: int = 4096) -> Table:
    """The star query with dimension filters lo <= f <= hi over every fact
    partition of `inputs`, its fact passes on `threads` host threads."""
    threads = threads or os.cpu_count() or 1
    lo = (ctypes.c_int32 * 4)(*[int(r[0]) for r in ranges])
    hi = (ctypes.c_int32 * 4)(*[int(r[1]) for r in ranges])
    g2 = np.zeros(max_groups, np.int32)
    g4 = np.zeros(max_groups, np.int32)
    rev = np.zeros(max_groups, np.int64)
    drev = np.zeros(max_groups, np.int64)
    cnt = np.zeros(max_groups, np.int64)
    n = lib().orc_star_query_parts(inputs.parts, inputs.n_parts, inputs.dims, lo, hi, bits, nh, threads,
                             g2.ctypes.data_as(ctypes.c_void_p), g4.ctypes.data_as(ctypes.c_void_p),
                             rev.ctypes.data_as(ctypes.c_void_p), drev.ctypes.data_as(ctypes.c_void_p),
                             cnt.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(max_groups))
    if n < 0:
        raise RuntimeError("too many groups")
    return Table([Column("d2_g", "int32", g2[:n]), Column("d4_g", "int32", g4[:n]),
                  Column("revenue", "int64", rev[:n]), Column("discount_revenue", "int64", drev[:n]),
                  Column("cnt", "int64", cnt[:n])])


def csv_scan(text: bytes, t_range, d1_lt: int, i1_lt: int, threads: int | None = None) -> tuple[int, int]:
    """(sum(d2 * i2), count) of the CSV scan workload, parsed by the C
    restatement on `threads` host threads."""
    threads = threads or os.cpu_count() or 1
    L = lib()
    L.orc_csv_scan.restype = ctypes.c_int64
    s = ctypes.c_int64()
    buf = ctypes.c_char_p(text)
    n = L.orc_csv_scan(buf, ctypes.c_int64(len(text)), ctypes.c_int64(t_range[0]), ctypes.c_int64(t_range[1]),
                       ctypes.c_int64(d1_lt), ctypes.c_int64(i1_lt), ctypes.c_int(threads), ctypes.byref(s))
    return s.value, n
