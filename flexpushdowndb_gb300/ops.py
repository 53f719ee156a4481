"""Python handles on the operator-level C ABI (one class per reference kernel).

These mirror the kernel seams of the reference's operators so tests read like
the reference's own: Filter (fpdb-expression-gandiva Filter::make / compile /
evaluate), BloomFilter (BloomFilterCreateArrowKernel / BloomFilterUseKernel),
HashJoin (HashJoinArrowKernel joinBuildTupleSet / finalizeInput /
joinProbeTupleSet), Group (GroupArrowKernel group / finalise) and csv_read
(CSVReader::read). Every call runs CUDA kernels inside libgfpdb.so.
"""

from __future__ import annotations

import ctypes
import json
from pathlib import Path
from typing import Sequence

import numpy as np

from . import _abi
from .expression import Expr, to_json
from .tupleset import DeviceTable, Exported, Table, export_host, import_result, new_output


def _export(t) -> Exported:
    if isinstance(t, Exported):
        return t
    if isinstance(t, DeviceTable):
        return t.export()
    if isinstance(t, Table):
        return export_host(t)
    raise TypeError(f"cannot export {type(t)}")


def _names(cols: Sequence[str] | None):
    if cols is None:
        return None, -1
    return _abi.cstr_array(list(cols)), len(cols)


def _key_list(k) -> list[str]:
    return [k] if isinstance(k, str) else list(k)


def init(device: int = 0) -> None:
    _abi.check(_abi.lib().gfpdb_device_init(device))


def kernel_launches() -> int:
    return int(_abi.lib().gfpdb_kernel_launch_count())


class Filter:
    """A compiled predicate (Filter::make + Filter::compile)."""

    def __init__(self, predicate: Expr, schema_of):
        self._h = ctypes.c_void_p()
        ex = _export(schema_of)
        _abi.check(_abi.lib().gfpdb_filter_compile(to_json(predicate).encode(), ex.schema_ptr, ctypes.byref(self._h)))

    def evaluate(self, table, project: Sequence[str] | None = None, stream=None) -> Table:
        ex = _export(table)
        names, n = _names(project)
        s, a = new_output()
        _abi.check(_abi.lib().gfpdb_filter_evaluate(self._h, ex.schema_ptr, ex.array_ptr, names, n, ctypes.byref(s),
                                                    ctypes.byref(a), stream))
        return import_result(s, a)

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            _abi.lib().gfpdb_filter_free(self._h)
            self._h = ctypes.c_void_p()


class BloomFilter:
    """Blocked bloom filter built on the device (BloomFilterCreateArrowKernel)."""

    def __init__(self, batches: Sequence, key_column: str | Sequence[str], bits_per_key: int = 10,
                 num_hashes: int = 3, stream=None):
        """key_column: one column name, or a list of them (the filter holds
        their composite)."""
        exs = [_export(b) for b in batches]
        if not exs:
            raise ValueError("BloomFilter needs at least one batch (the schema comes from it)")
        arr = (ctypes.POINTER(_abi.ArrowDeviceArray) * len(exs))(*[e.array_ptr for e in exs])
        keys = _key_list(key_column)
        self._h = ctypes.c_void_p()
        _abi.check(_abi.lib().gfpdb_bloom_create(exs[0].schema_ptr, arr, len(exs), _abi.cstr_array(keys), len(keys),
                                                 bits_per_key, num_hashes, ctypes.byref(self._h), stream))

    def info(self) -> dict:
        nb, nk = ctypes.c_int64(), ctypes.c_int64()
        valid, nh = ctypes.c_int32(), ctypes.c_int32()
        ptr = ctypes.c_void_p()
        _abi.check(_abi.lib().gfpdb_bloom_info(self._h, ctypes.byref(nb), ctypes.byref(nk), ctypes.byref(valid),
                                               ctypes.byref(nh), ctypes.byref(ptr)))
        return {"num_blocks": nb.value, "num_keys": nk.value, "valid": bool(valid.value), "num_hashes": nh.value,
                "device_ptr": ptr.value}

    def words(self) -> np.ndarray:
        """The filter's uint32 words, copied to the host."""
        info = self.info()
        out = np.zeros(info["num_blocks"] * 8, dtype=np.uint32)
        if out.nbytes:
            _abi.check(_abi.lib().gfpdb_memcpy(out.ctypes.data, info["device_ptr"], out.nbytes, 2, None))
        return out

    def use(self, table, key_column: str | Sequence[str], stream=None) -> Table:
        ex = _export(table)
        keys = _key_list(key_column)
        s, a = new_output()
        _abi.check(_abi.lib().gfpdb_bloom_use(self._h, ex.schema_ptr, ex.array_ptr, _abi.cstr_array(keys), len(keys),
                                              ctypes.byref(s), ctypes.byref(a), stream))
        return import_result(s, a)

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            _abi.lib().gfpdb_bloom_free(self._h)
            self._h = ctypes.c_void_p()


def shuffle(table, key_columns: str | Sequence[str], num_slots: int, stream=None) -> tuple[Table, list[int]]:
    """Hash-partition the rows into num_slots slots (gfpdb_shuffle,
    ShuffleKernel2::shuffle): the rows slot by slot, and the num_slots + 1
    slot offsets."""
    ex = _export(table)
    keys = _key_list(key_columns)
    offs = (ctypes.c_int64 * (num_slots + 1))()
    s, a = new_output()
    _abi.check(_abi.lib().gfpdb_shuffle(ex.schema_ptr, ex.array_ptr, _abi.cstr_array(keys), len(keys), num_slots,
                                        ctypes.byref(s), ctypes.byref(a), offs, stream))
    return import_result(s, a), list(offs)


def shuffle_split(table, key_columns: str | Sequence[str], num_slots: int, stream=None) -> list[Table]:
    """The same as one Table per slot (the reference's vector of TupleSets)."""
    rows, offs = shuffle(table, key_columns, num_slots, stream)
    return [rows.slice(offs[i], offs[i + 1]) for i in range(num_slots)]


def select(table, predicate: Filter | None = None, blooms: Sequence[tuple[BloomFilter, str]] = (),
           project: Sequence[str] | None = None, stream=None) -> Table:
    """Fused predicate + bloom probes + compaction (gfpdb_select)."""
    ex = _export(table)
    nb = len(blooms)
    bh = (ctypes.c_void_p * max(1, nb))(*[b._h.value for b, _ in blooms])
    bc = _abi.cstr_array([c for _, c in blooms])
    names, n = _names(project)
    s, a = new_output()
    _abi.check(_abi.lib().gfpdb_select(predicate._h if predicate else None, nb, bh, bc, ex.schema_ptr, ex.array_ptr,
                                       names, n, ctypes.byref(s), ctypes.byref(a), stream))
    return import_result(s, a)


JOIN_TYPES = {"INNER": 0, "LEFT": 1, "RIGHT": 2, "FULL": 3, "LEFT_SEMI": 4, "RIGHT_SEMI": 5}


class HashJoin:
    """Hash join (HashJoinArrowKernel). Output: probe columns, then build
    columns (one side only for semi joins)."""

    def __init__(self, build_key: str | Sequence[str], probe_key: str | Sequence[str],
                 needed: Sequence[str] | None = None, load_factor: float = 0.5, join_type: str = "INNER"):
        """Keys: one column per side, or equally long lists (build_key[i]
        matches probe_key[i]). join_type: the reference's JoinType (LEFT
        keeps every build row, RIGHT every probe row; the rows the build side
        decides come from finish())."""
        names, n = _names(needed)
        bk, pk = _key_list(build_key), _key_list(probe_key)
        if len(bk) != len(pk):
            raise ValueError("as many probe key columns as build key columns")
        self._h = ctypes.c_void_p()
        _abi.check(_abi.lib().gfpdb_hashjoin_create(JOIN_TYPES[join_type], _abi.cstr_array(bk), _abi.cstr_array(pk),
                                                    len(bk), names, n, load_factor, ctypes.byref(self._h)))

    def put_build(self, table, stream=None) -> None:
        ex = _export(table)
        _abi.check(_abi.lib().gfpdb_hashjoin_put_build(self._h, ex.schema_ptr, ex.array_ptr, stream))

    def finalize_build(self, stream=None) -> None:
        _abi.check(_abi.lib().gfpdb_hashjoin_finalize_build(self._h, stream))

    def probe(self, table, stream=None) -> Table:
        ex = _export(table)
        s, a = new_output()
        _abi.check(_abi.lib().gfpdb_hashjoin_probe(self._h, ex.schema_ptr, ex.array_ptr, ctypes.byref(s),
                                                   ctypes.byref(a), stream))
        return import_result(s, a)

    def finish(self, probe_schema_of=None, stream=None) -> Table:
        """The rows the build side decides once every probe batch is in
        (LEFT / FULL: unmatched build rows, LEFT_SEMI: matched ones)."""
        ex = _export(probe_schema_of) if probe_schema_of is not None else None
        s, a = new_output()
        _abi.check(_abi.lib().gfpdb_hashjoin_finish(self._h, ex.schema_ptr if ex else None, ctypes.byref(s),
                                                    ctypes.byref(a), stream))
        return import_result(s, a)

    def clear(self) -> None:
        """Drop the build side and the table (HashJoinArrowKernel::clear)."""
        _abi.check(_abi.lib().gfpdb_hashjoin_clear(self._h))

    def info(self) -> dict:
        b, c, m = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _abi.check(_abi.lib().gfpdb_hashjoin_info(self._h, ctypes.byref(b), ctypes.byref(c), ctypes.byref(m)))
        return {"build_rows": b.value, "capacity": c.value, "max_probe": m.value}

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            _abi.lib().gfpdb_hashjoin_free(self._h)
            self._h = ctypes.c_void_p()


def aggregate(function: str, name: str, expr: Expr | None = None) -> dict:
    a = {"function": function, "name": name}
    if expr is not None:
        a["expr"] = expr
    return a


class Group:
    """Hash group-by (GroupArrowKernel): group() per TupleSet, finalise() once."""

    def __init__(self, group_columns: Sequence[str], aggregates: Sequence[dict], groups_hint: int = 0):
        spec = {"groupColumnNames": list(group_columns), "aggregates": list(aggregates), "groupsHint": groups_hint}
        self._h = ctypes.c_void_p()
        _abi.check(_abi.lib().gfpdb_group_create(json.dumps(spec).encode(), ctypes.byref(self._h)))

    def group(self, table, stream=None) -> None:
        ex = _export(table)
        _abi.check(_abi.lib().gfpdb_group_update(self._h, ex.schema_ptr, ex.array_ptr, stream))

    def clear(self) -> None:
        """Drop every group (GroupAbstractKernel::clear)."""
        _abi.check(_abi.lib().gfpdb_group_clear(self._h))

    def finalise(self, stream=None) -> Table:
        s, a = new_output()
        _abi.check(_abi.lib().gfpdb_group_finalize(self._h, ctypes.byref(s), ctypes.byref(a), stream))
        return import_result(s, a)

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            _abi.lib().gfpdb_group_free(self._h)
            self._h = ctypes.c_void_p()


def parquet_read(source, columns: Sequence[str] | None = None, start_pos: int = 0, end_pos: int = -1,
                 stream=None) -> Table:
    """Read columns of a Parquet file (gfpdb_parquet_read / _read_file,
    ParquetReader::read, readRange when start_pos <= end_pos): `source` is
    the file's bytes or a path of the local file system."""
    names, n = _names(columns)
    s, a = new_output()
    L = _abi.lib()
    if isinstance(source, (str, Path)):
        _abi.check(L.gfpdb_parquet_read_file(str(source).encode(), names, n, start_pos, end_pos, ctypes.byref(s),
                                             ctypes.byref(a), stream))
    else:
        buf = np.frombuffer(source, dtype=np.uint8) if isinstance(source, (bytes, bytearray)) else source
        _abi.check(L.gfpdb_parquet_read(buf.ctypes.data, buf.nbytes, names, n, start_pos, end_pos, ctypes.byref(s),
                                        ctypes.byref(a), stream))
    return import_result(s, a)


def parquet_layout(source, columns: Sequence[str] | None = None, start_pos: int = 0, end_pos: int = -1) -> dict:
    """The columns, row groups, column chunks and pages of a Parquet file
    that parquet_read with the same arguments reads (gfpdb_parquet_layout,
    host only); `source` is the file's bytes or a path."""
    import json

    if isinstance(source, (str, Path)):
        source = Path(source).read_bytes()
    buf = np.frombuffer(source, dtype=np.uint8) if isinstance(source, (bytes, bytearray)) else source
    names, n = _names(columns)
    L = _abi.lib()
    need = ctypes.c_int64()
    rc = L.gfpdb_parquet_layout(buf.ctypes.data, buf.nbytes, names, n, start_pos, end_pos, None, 0,
                                ctypes.byref(need))
    if need.value <= 0:
        _abi.check(rc)
    out = ctypes.create_string_buffer(need.value)
    _abi.check(L.gfpdb_parquet_layout(buf.ctypes.data, buf.nbytes, names, n, start_pos, end_pos, out, need.value,
                                      ctypes.byref(need)))
    return json.loads(out.value.decode())


def csv_read(text: bytes | np.ndarray | int, fields: Sequence[tuple[str, str]], columns: Sequence[str] | None = None,
             delimiter: str = ",", has_header: bool = False, device_ptr: int | None = None, stream=None,
             to_host: bool = True):
    """Parse delimited text (CSVReader::read). ``fields`` lists (name, type)
    for every field of a line; a type "decimal(p,s)" parses into int64
    scaled by 10^s. With device_ptr, `text` is the byte count of device text.
    With to_host False the parsed columns stay on the device and are
    released; the row count is returned (for timing the ingest alone)."""
    schema_children = []
    for name, ty in fields:
        if ty.startswith("decimal"):
            inner = ty[ty.index("(") + 1 : ty.index(")")]
            schema_children.append((name, ("d:" + inner.replace(" ", "")).encode()))
        else:
            from .tupleset import FORMATS

            schema_children.append((name, FORMATS[ty]))
    keep = []
    kids = (_abi.ArrowSchema * len(schema_children))()
    kid_ptrs = (ctypes.POINTER(_abi.ArrowSchema) * len(schema_children))()
    from .tupleset import _noop_schema_release

    for i, (name, fmt) in enumerate(schema_children):
        bn = name.encode()
        keep += [bn, fmt]
        kids[i].format = fmt
        kids[i].name = bn
        kids[i].release = _noop_schema_release
        kid_ptrs[i] = ctypes.pointer(kids[i])
    sch = _abi.ArrowSchema()
    sch.format = b"+s"
    sch.n_children = len(schema_children)
    sch.children = ctypes.cast(kid_ptrs, ctypes.POINTER(ctypes.POINTER(_abi.ArrowSchema)))
    sch.release = _noop_schema_release
    names, n = _names(columns)
    s, a = new_output()
    if device_ptr is not None:
        nbytes = len(text) if not isinstance(text, int) else text
        ptr, dev_type = device_ptr, _abi.ARROW_DEVICE_CUDA
    else:
        buf = np.frombuffer(text, dtype=np.uint8) if isinstance(text, (bytes, bytearray)) else text
        keep.append(buf)
        nbytes, ptr, dev_type = buf.nbytes, buf.ctypes.data, _abi.ARROW_DEVICE_CPU
    _abi.check(_abi.lib().gfpdb_csv_read(ptr, nbytes, dev_type, delimiter.encode(), 1 if has_header else 0,
                                         ctypes.byref(sch), names, n, ctypes.byref(s), ctypes.byref(a), stream))
    if not to_host:
        from .tupleset import release_result

        return release_result(s, a)
    return import_result(s, a)
