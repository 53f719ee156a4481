"""A small Parquet writer: Tables to Parquet bytes, written to the public
Apache Parquet format (parquet.thrift's FileMetaData, RowGroup, ColumnChunk,
ColumnMetaData and PageHeader in the Thrift compact protocol). Flat REQUIRED
columns (int32, int64, float64, date32, utf8), data pages v1, no
compression; each column chunk PLAIN, or dictionary-encoded (a PLAIN
dictionary page, then data pages of bit-packed indices) when it has few
distinct values. It makes large Parquet inputs for the reader's measurements
where no other writer is installed; any Parquet reader reads its files.
"""

from __future__ import annotations

import struct

import numpy as np

from .tupleset import Table

_PT = {"int32": 1, "int64": 2, "float64": 5, "date32": 1, "utf8": 6}  # physical types
_CONVERTED = {"utf8": 0, "date32": 6}  # ConvertedType UTF8, DATE


class _Compact:
    """Thrift compact protocol writer."""

    def __init__(self):
        self.out = bytearray()
        self.last = [0]

    def varint(self, v: int):
        while True:
            b = v & 0x7F
            v >>= 7
            if v:
                self.out.append(b | 0x80)
            else:
                self.out.append(b)
                return

    def zigzag(self, v: int):
        self.varint((v << 1) ^ (v >> 63))

    def field(self, fid: int, ftype: int):
        delta = fid - self.last[-1]
        if 0 < delta <= 15:
            self.out.append((delta << 4) | ftype)
        else:
            self.out.append(ftype)
            self.zigzag(fid)
        self.last[-1] = fid

    def i32(self, fid, v):
        self.field(fid, 5)
        self.zigzag(v)

    def i64(self, fid, v):
        self.field(fid, 6)
        self.zigzag(v)

    def binary(self, fid, b: bytes):
        self.field(fid, 8)
        self.varint(len(b))
        self.out += b

    def begin_struct(self, fid):
        self.field(fid, 12)
        self.last.append(0)

    def end_struct(self):
        self.out.append(0)
        self.last.pop()

    def list_header(self, fid, etype, n):
        self.field(fid, 9)
        if n < 15:
            self.out.append((n << 4) | etype)
        else:
            self.out.append(0xF0 | etype)
            self.varint(n)

    def list_struct_begin(self):
        self.last.append(0)


def _plain(ty: str, values) -> bytes:
    if ty == "utf8":
        parts = []
        for s in values:
            b = s.encode() if isinstance(s, str) else bytes(s)
            parts.append(struct.pack("<i", len(b)) + b)
        return b"".join(parts)
    dt = {"int32": "<i4", "date32": "<i4", "int64": "<i8", "float64": "<f8"}[ty]
    return np.ascontiguousarray(values, dtype=dt).tobytes()


def _bitpacked(idx: np.ndarray, bw: int) -> bytes:
    """One bit-packed run of the RLE / bit-packed hybrid (the values padded
    to a multiple of 8), behind its bit-width byte."""
    n = len(idx)
    groups = (n + 7) // 8
    padded = np.zeros(groups * 8, dtype=np.uint32)
    padded[:n] = idx
    bits = ((padded[:, None] >> np.arange(bw, dtype=np.uint32)) & 1).astype(np.uint8).reshape(-1)
    w = _Compact()
    w.varint((groups << 1) | 1)
    return bytes([bw]) + bytes(w.out) + np.packbits(bits, bitorder="little").tobytes()


def _page_header(page_type: int, size: int, num_values: int, encoding: int) -> bytes:
    w = _Compact()
    w.i32(1, page_type)
    w.i32(2, size)
    w.i32(3, size)
    if page_type == 2:  # dictionary page
        w.begin_struct(7)
        w.i32(1, num_values)
        w.i32(2, 0)  # PLAIN
        w.end_struct()
    else:
        w.begin_struct(5)
        w.i32(1, num_values)
        w.i32(2, encoding)
        w.i32(3, 3)  # definition levels: RLE (none written: REQUIRED columns)
        w.i32(4, 3)
        w.end_struct()
    w.out.append(0)
    return bytes(w.out)


def write_parquet(table: Table, row_group_rows: int = 1 << 20, page_rows: int = 1 << 16,
                  dictionary_max: int = 1 << 15) -> bytes:
    """The table as a Parquet file's bytes. A column chunk with at most
    `dictionary_max` distinct values is dictionary-encoded."""
    out = bytearray(b"PAR1")
    n = table.num_rows
    groups = []
    strings = {c.name: c.to_list() for c in table.columns if c.type == "utf8"}
    for g0 in range(0, max(n, 1), row_group_rows):
        g1 = min(n, g0 + row_group_rows)
        chunks = []
        for c in table.columns:
            vals = strings[c.name][g0:g1] if c.type == "utf8" else c.values[g0:g1]
            start = len(out)
            dict_off = None
            encodings = [0, 3]
            uniq = None
            if dictionary_max > 0 and g1 > g0:
                if c.type == "utf8":
                    keys = {}
                    codes = np.fromiter((keys.setdefault(v, len(keys)) for v in vals), dtype=np.int64, count=len(vals))
                    if len(keys) <= dictionary_max:
                        uniq = list(keys)
                else:
                    u, inv = np.unique(np.asarray(vals), return_inverse=True)
                    if len(u) <= dictionary_max:
                        uniq, codes = u, inv
            if uniq is not None:
                body = _plain(c.type, uniq)
                dict_off = len(out)
                out += _page_header(2, len(body), len(uniq), 0) + body
                encodings = [0, 3, 8]
            data_off = len(out)
            for p0 in range(g0, g1, page_rows):
                p1 = min(g1, p0 + page_rows)
                if uniq is not None:
                    bw = max(1, int(len(uniq) - 1).bit_length())
                    body = _bitpacked(np.asarray(codes[p0 - g0 : p1 - g0], dtype=np.uint32), bw)
                    enc = 8  # RLE_DICTIONARY
                else:
                    body = _plain(c.type, vals[p0 - g0 : p1 - g0])
                    enc = 0
                out += _page_header(0, len(body), p1 - p0, enc) + body
            if g1 == g0:  # an empty table: one empty page
                out += _page_header(0, 0, 0, 0)
            chunks.append((c, start, dict_off, data_off, len(out) - start, encodings))
        groups.append((g1 - g0, chunks))

    w = _Compact()
    w.i32(1, 1)
    w.list_header(2, 12, 1 + len(table.columns))
    w.list_struct_begin()
    w.binary(4, b"schema")
    w.i32(5, len(table.columns))
    w.out.append(0)
    for c in table.columns:
        w.last[-1] = 0
        w.i32(1, _PT[c.type])
        w.i32(3, 0)  # REQUIRED
        w.binary(4, c.name.encode())
        if c.type in _CONVERTED:
            w.i32(6, _CONVERTED[c.type])
        w.out.append(0)
    w.last.pop()
    w.i64(3, n)
    w.list_header(4, 12, len(groups))
    w.list_struct_begin()
    for rows, chunks in groups:
        w.last[-1] = 0
        w.list_header(1, 12, len(chunks))
        w.list_struct_begin()
        total = 0
        for c, start, dict_off, data_off, size, encodings in chunks:
            w.last[-1] = 0
            w.i64(2, start)
            w.begin_struct(3)
            w.i32(1, _PT[c.type])
            w.list_header(2, 5, len(encodings))
            for e in encodings:
                w.zigzag(e)
            w.list_header(3, 8, 1)
            nb = c.name.encode()
            w.varint(len(nb))
            w.out += nb
            w.i32(4, 0)  # UNCOMPRESSED
            w.i64(5, rows)
            w.i64(6, size)
            w.i64(7, size)
            w.i64(9, data_off)
            if dict_off is not None:
                w.i64(11, dict_off)
            w.end_struct()
            w.out.append(0)
            total += size
        w.last.pop()
        w.i64(2, total)
        w.i64(3, rows)
        w.out.append(0)
    w.last.pop()
    w.binary(6, b"flexpushdowndb_gb300 parquet_writer")
    w.out.append(0)
    out += w.out
    out += struct.pack("<I", len(w.out)) + b"PAR1"
    return bytes(out)
