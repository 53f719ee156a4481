"""Host-side TupleSet values and their Arrow C Data Interface form.

``Table`` is a host (numpy) TupleSet used to hand inputs to the library and
to read its results back; ``DeviceTable`` holds the same columns in device
memory (torch tensors are used only as device allocations). Both export to
the (ArrowSchema "+s", ArrowDeviceArray) pair the C ABI takes; results come
back through ``import_result``.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Any, Iterable, Sequence

import numpy as np

from . import _abi

FORMATS = {"int32": b"i", "int64": b"l", "date32": b"tdD", "float64": b"g", "utf8": b"u"}
TYPES = {v: k for k, v in FORMATS.items()}
NP_TYPES = {"int32": np.int32, "int64": np.int64, "date32": np.int32, "float64": np.float64}


def utf8_encode(values: Sequence[str | bytes]) -> tuple[np.ndarray, np.ndarray]:
    """List of strings -> (int32 offsets, uint8 bytes)."""
    enc = [v.encode() if isinstance(v, str) else bytes(v) for v in values]
    lens = np.fromiter((len(b) for b in enc), dtype=np.int64, count=len(enc))
    offs = np.zeros(len(enc) + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    if offs[-1] > np.iinfo(np.int32).max:
        raise ValueError("utf8 column exceeds 2 GiB")
    data = np.frombuffer(b"".join(enc), dtype=np.uint8).copy()
    return offs.astype(np.int32), data


def utf8_decode(offsets: np.ndarray, data: np.ndarray) -> list[str]:
    raw = data.tobytes()
    o = offsets.astype(np.int64)
    return [raw[o[i] : o[i + 1]].decode() for i in range(len(o) - 1)]


@dataclass
class Column:
    name: str
    type: str
    values: Any  # np.ndarray (fixed width) or (offsets, bytes) for utf8
    valid: Any = None  # None (no nulls) or a bool array, False at a null

    def __post_init__(self):
        if self.type not in FORMATS:
            raise ValueError(f"unsupported type {self.type}")
        if self.type == "utf8":
            if not isinstance(self.values, tuple):
                self.values = utf8_encode(list(self.values))
        else:
            self.values = np.ascontiguousarray(self.values, dtype=NP_TYPES[self.type])

    def __len__(self) -> int:
        return len(self.values[0]) - 1 if self.type == "utf8" else len(self.values)

    def to_list(self) -> list:
        vals = utf8_decode(*self.values) if self.type == "utf8" else self.values.tolist()
        if self.valid is not None:
            vals = [v if ok else None for v, ok in zip(vals, self.valid.tolist())]
        return vals


class Table:
    """An ordered set of equal-length host columns."""

    def __init__(self, columns: Iterable[Column]):
        self.columns = list(columns)
        lens = {len(c) for c in self.columns}
        if len(lens) > 1:
            raise ValueError(f"ragged table: column lengths {lens}")

    @classmethod
    def from_dict(cls, cols: dict[str, tuple[str, Any]]) -> "Table":
        return cls(Column(n, t, v) for n, (t, v) in cols.items())

    @property
    def num_rows(self) -> int:
        return len(self.columns[0]) if self.columns else 0

    @property
    def names(self) -> list[str]:
        return [c.name for c in self.columns]

    def column(self, name: str) -> Column:
        for c in self.columns:
            if c.name == name:
                return c
        raise KeyError(name)

    def __getitem__(self, name: str):
        c = self.column(name)
        return c.to_list() if c.type == "utf8" else c.values

    def rows(self) -> list[tuple]:
        cols = [c.to_list() for c in self.columns]
        return list(zip(*cols)) if cols else []

    def sorted_rows(self) -> list[tuple]:
        """Rows as a sorted multiset (join and group outputs have no order);
        nulls sort after values."""
        return sorted(self.rows(), key=lambda r: tuple((v is None, 0 if v is None else v) for v in r))

    def nbytes(self) -> int:
        n = 0
        for c in self.columns:
            n += c.values[0].nbytes + c.values[1].nbytes if c.type == "utf8" else c.values.nbytes
        return n

    @staticmethod
    def concat(tables: Sequence["Table"]) -> "Table":
        """Row-wise concatenation of tables with the same columns."""
        cols = []
        for i, c in enumerate(tables[0].columns):
            parts = [t.columns[i] for t in tables]
            if c.type == "utf8":
                cols.append(Column(c.name, c.type, sum((p.to_list() for p in parts), [])))
            else:
                cols.append(Column(c.name, c.type, np.concatenate([p.values for p in parts])))
        return Table(cols)

    def slice(self, start: int, stop: int) -> "Table":
        out = []
        for c in self.columns:
            if c.type == "utf8":
                o, d = c.values
                lo, hi = int(o[start]), int(o[stop])
                out.append(Column(c.name, c.type, ((o[start : stop + 1] - lo).astype(np.int32), d[lo:hi].copy())))
            else:
                out.append(Column(c.name, c.type, c.values[start:stop]))
            if c.valid is not None:
                out[-1].valid = c.valid[start:stop]
        return Table(out)


# ---------------------------------------------------------------- export


@_abi.SCHEMA_RELEASE
def _noop_schema_release(ptr):
    ptr.contents.release = _abi.SCHEMA_RELEASE()


@_abi.ARRAY_RELEASE
def _noop_array_release(ptr):
    ptr.contents.release = _abi.ARRAY_RELEASE()


@dataclass
class Exported:
    """Arrow C structures describing a table; keeps every buffer alive."""

    schema: _abi.ArrowSchema
    array: _abi.ArrowDeviceArray
    keep: list = field(default_factory=list)

    @property
    def schema_ptr(self):
        return ctypes.pointer(self.schema)

    @property
    def array_ptr(self):
        return ctypes.pointer(self.array)


def _export(names, types, buffers_per_col, length, device_type, device_id) -> Exported:
    keep: list = []
    n = len(names)
    child_schemas = (_abi.ArrowSchema * max(1, n))()
    child_schema_ptrs = (ctypes.POINTER(_abi.ArrowSchema) * max(1, n))()
    child_arrays = (_abi.ArrowArray * max(1, n))()
    child_array_ptrs = (ctypes.POINTER(_abi.ArrowArray) * max(1, n))()
    for i, (nm, ty, bufs) in enumerate(zip(names, types, buffers_per_col)):
        bname = nm.encode()
        keep.append(bname)
        cs = child_schemas[i]
        cs.format = FORMATS[ty]
        cs.name = bname
        cs.release = _noop_schema_release
        child_schema_ptrs[i] = ctypes.pointer(cs)
        bufarr = (ctypes.c_void_p * len(bufs))(*bufs)
        keep.append(bufarr)
        ca = child_arrays[i]
        ca.length = length
        ca.null_count = 0
        ca.offset = 0
        ca.n_buffers = len(bufs)
        ca.buffers = ctypes.cast(bufarr, ctypes.POINTER(ctypes.c_void_p))
        ca.release = _noop_array_release
        child_array_ptrs[i] = ctypes.pointer(ca)
    keep += [child_schemas, child_schema_ptrs, child_arrays, child_array_ptrs]
    schema = _abi.ArrowSchema()
    schema.format = b"+s"
    schema.name = b""
    schema.n_children = n
    schema.children = ctypes.cast(child_schema_ptrs, ctypes.POINTER(ctypes.POINTER(_abi.ArrowSchema)))
    schema.release = _noop_schema_release
    top_bufs = (ctypes.c_void_p * 1)(None)
    keep.append(top_bufs)
    arr = _abi.ArrowDeviceArray()
    arr.array.length = length
    arr.array.null_count = 0
    arr.array.offset = 0
    arr.array.n_buffers = 1
    arr.array.buffers = ctypes.cast(top_bufs, ctypes.POINTER(ctypes.c_void_p))
    arr.array.n_children = n
    arr.array.children = ctypes.cast(child_array_ptrs, ctypes.POINTER(ctypes.POINTER(_abi.ArrowArray)))
    arr.array.release = _noop_array_release
    arr.device_type = device_type
    arr.device_id = device_id
    return Exported(schema, arr, keep)


def export_host(table: Table, pinned: bool = False) -> Exported:
    """Export host columns. With ``pinned`` the values are first copied into
    page-locked memory (so host-to-device copies run at link speed)."""
    bufs_per_col = []
    keep = []
    for c in table.columns:
        arrays = list(c.values) if c.type == "utf8" else [c.values]
        ptrs: list = [None]
        for a in arrays:
            if pinned:
                h = PinnedBuffer(a.nbytes)
                h.view(a.dtype, a.shape)[...] = a
                keep.append(h)
                ptrs.append(h.ptr)
            else:
                keep.append(a)
                ptrs.append(a.ctypes.data if a.nbytes else None)
        bufs_per_col.append(ptrs)
    ex = _export(table.names, [c.type for c in table.columns], bufs_per_col, table.num_rows,
                 _abi.ARROW_DEVICE_CUDA_HOST if pinned else _abi.ARROW_DEVICE_CPU, -1)
    ex.keep += keep
    return ex


class PinnedBuffer:
    """Page-locked host memory from gfpdb_host_alloc."""

    def __init__(self, nbytes: int):
        p = ctypes.c_void_p()
        _abi.check(_abi.lib().gfpdb_host_alloc(ctypes.byref(p), max(1, nbytes)))
        self.ptr = p.value
        self.nbytes = nbytes

    def view(self, dtype, shape) -> np.ndarray:
        buf = (ctypes.c_char * max(1, self.nbytes)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape)) if shape else 1).reshape(shape)

    def __del__(self):
        try:
            if self.ptr:
                _abi.lib().gfpdb_host_free(self.ptr)
        except Exception:
            pass


class DeviceTable:
    """Columns resident in device memory (torch tensors as allocations)."""

    def __init__(self, names, types, tensors, num_rows):
        self.names = names
        self.types = types
        self.tensors = tensors  # per column: [values] or [offsets, bytes]
        self.num_rows = num_rows

    @classmethod
    def from_host(cls, table: Table, device: str = "cuda") -> "DeviceTable":
        import torch

        tensors = []
        for c in table.columns:
            arrays = list(c.values) if c.type == "utf8" else [c.values]
            tensors.append([torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in arrays])
        return cls(table.names, [c.type for c in table.columns], tensors, table.num_rows)

    def export(self) -> Exported:
        import torch

        bufs = [[None] + [t.data_ptr() for t in ts] for ts in self.tensors]
        dev = torch.cuda.current_device()
        ex = _export(self.names, self.types, bufs, self.num_rows, _abi.ARROW_DEVICE_CUDA, dev)
        ex.keep.append(self)
        return ex

    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for ts in self.tensors for t in ts)


def new_output() -> tuple[_abi.ArrowSchema, _abi.ArrowDeviceArray]:
    return _abi.ArrowSchema(), _abi.ArrowDeviceArray()


def release_result(schema: _abi.ArrowSchema, darr: _abi.ArrowDeviceArray) -> int:
    """Release an exported TupleSet without copying it; returns its rows."""
    n = darr.array.length
    if darr.array.release:
        darr.array.release(ctypes.pointer(darr.array))
    if schema.release:
        schema.release(ctypes.pointer(schema))
    return n


def import_result(schema: _abi.ArrowSchema, darr: _abi.ArrowDeviceArray, release: bool = True) -> Table:
    """Copy an exported TupleSet (device or host) into a host Table and
    release the library's structures."""
    L = _abi.lib()
    n = darr.array.length
    on_device = darr.device_type == _abi.ARROW_DEVICE_CUDA
    cols = []

    def fetch(ptr, nbytes, dtype):
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype=dtype)
        if nbytes == 0:
            return out
        if on_device:
            _abi.check(L.gfpdb_memcpy(out.ctypes.data, ptr, nbytes, 2, None))
        else:
            ctypes.memmove(out.ctypes.data, ptr, nbytes)
        return out

    for i in range(schema.n_children):
        cs = schema.children[i].contents
        ca = darr.array.children[i].contents
        ty = TYPES[cs.format]
        name = cs.name.decode()
        if ty == "utf8":
            offs = fetch(ca.buffers[1], (n + 1) * 4, np.int32)
            base = int(offs[0]) if n >= 0 and len(offs) else 0
            total = int(offs[-1]) - base if len(offs) else 0
            data = np.empty(0, dtype=np.uint8)
            if total > 0:
                raw = np.empty(total, dtype=np.uint8)
                src = ca.buffers[2] + base
                if on_device:
                    _abi.check(L.gfpdb_memcpy(raw.ctypes.data, src, total, 2, None))
                else:
                    ctypes.memmove(raw.ctypes.data, src, total)
                data = raw
            cols.append(Column(name, ty, ((offs - base).astype(np.int32), data)))
        else:
            dt = NP_TYPES[ty]
            cols.append(Column(name, ty, fetch(ca.buffers[1], n * np.dtype(dt).itemsize, dt)))
        if ca.buffers[0] and ca.null_count != 0:
            bits = fetch(ca.buffers[0], (n + 7) // 8, np.uint8)
            cols[-1].valid = np.unpackbits(bits, bitorder="little")[:n].astype(bool)
    if release:
        if darr.array.release:
            darr.array.release(ctypes.pointer(darr.array))
        if schema.release:
            schema.release(ctypes.pointer(schema))
    return Table(cols)


class ResultReader:
    """Copies exported TupleSets into host Tables with one layout call and one
    release call into the library (instead of walking the Arrow structures
    field by field through ctypes), reusing its argument buffers: the import
    for a loop that reads many results."""

    MAX_COLUMNS = 256
    NAMES_BYTES = 1 << 16

    def __init__(self):
        L = _abi.lib()
        self._layout = L.gfpdb_result_layout
        self._release = L.gfpdb_result_release
        self._memcpy = L.gfpdb_memcpy
        self._n, self._nc, self._dev = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
        self._refs = (ctypes.byref(self._n), ctypes.byref(self._nc), ctypes.byref(self._dev))
        self._names = ctypes.create_string_buffer(self.NAMES_BYTES)
        self._vals = (ctypes.c_void_p * self.MAX_COLUMNS)()
        self._offs = (ctypes.c_void_p * self.MAX_COLUMNS)()

    def _copy(self, dst: np.ndarray, src: int, nbytes: int, on_device: bool) -> None:
        if nbytes == 0:
            return
        if on_device:
            _abi.check(self._memcpy(dst.ctypes.data, src, nbytes, 2, None))
        else:
            ctypes.memmove(dst.ctypes.data, src, nbytes)

    def read(self, schema: _abi.ArrowSchema, darr: _abi.ArrowDeviceArray) -> Table:
        sref, aref = ctypes.byref(schema), ctypes.byref(darr)
        try:
            _abi.check(self._layout(sref, aref, self.MAX_COLUMNS, *self._refs, self._names, self.NAMES_BYTES,
                                    self._vals, self._offs))
            n, nc = self._n.value, self._nc.value
            on_device = self._dev.value == _abi.ARROW_DEVICE_CUDA
            parts = self._names.raw.split(b"\0", 2 * nc)
            cols = []
            for i in range(nc):
                ty = TYPES[parts[2 * i + 1]]
                if ty == "utf8":
                    offs = np.empty(n + 1, dtype=np.int32)
                    self._copy(offs, self._offs[i], (n + 1) * 4, on_device)
                    base = int(offs[0])
                    data = np.empty(int(offs[-1]) - base, dtype=np.uint8)
                    self._copy(data, self._vals[i] + base, data.nbytes, on_device)
                    values = ((offs - base).astype(np.int32), data)
                else:
                    values = np.empty(n, dtype=NP_TYPES[ty])
                    self._copy(values, self._vals[i], values.nbytes, on_device)
                c = Column.__new__(Column)  # the values already have the column's dtype and layout
                c.name, c.type, c.values = parts[2 * i].decode(), ty, values
                cols.append(c)
            return Table(cols)
        finally:
            self._release(sref, aref)


def text_table(text: bytes, name: str = "text") -> Table:
    """A one-row table whose utf8 value is `text` (the input of CsvScanPOp)."""
    if len(text) >= 2**31:
        raise ValueError("text exceeds 2 GiB")
    return Table([Column(name, "utf8", (np.array([0, len(text)], dtype=np.int32), np.frombuffer(text, dtype=np.uint8)))])
