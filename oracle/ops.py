"""Operator restatements on numpy (TEST INFRASTRUCTURE ONLY).

Each function follows the reference operator it names:
  filter_table  - Filter::evaluate (fpdb-expression-gandiva/src/Filter.cpp:87-225):
                  rows where the predicate is true, input order kept, then
                  the projection.
  bloom_*       - the 256-bit-block bloom design of this project (the
                  reference's bloom is Arrow's, vendored in
                  fpdb-tuple/src/arrow/exec/BloomFilter.cpp, and its
                  Carter-Wegman variant draws random hash functions, so only
                  "no false negatives" is shared with it; the bit array here is
                  the exact expected content of the device filter).
  hash_join_typed - the INNER / LEFT / RIGHT / FULL / LEFT_SEMI / RIGHT_SEMI
                  joins with the reference's sides (below), nulls as a
                  validity mask.
  hash_join     - inner join, output probe columns then build columns
                  (HashJoinArrowKernel::makeOutputSchema,
                  fpdb-executor/src/physical/join/hashjoin/HashJoinArrowKernel.cpp:148-162),
                  every (probe, build) key match emitted.
  group_by      - hash_sum (int64 two's-complement wrapping sums) /
                  hash_count / min / max / avg per group, output group
                  columns then aggregates (GroupArrowKernel.cpp:156-200,
                  Sum.cpp:63-74, Count.cpp:91-104).
  csv_parse     - CSVToArrowSIMDChunkParser.cpp:183-374 field rules, with
                  decimals as exact scaled int64 and dates as date32.
  project       - ProjectPOp::projectAndSendTuples
                  (fpdb-executor/src/physical/project/ProjectPOp.cpp:98-145):
                  the renamed pass-through columns, then one column per
                  expression.
  shuffle       - ShuffleKernel2::shuffle
                  (fpdb-executor/src/physical/shuffle/ShuffleKernel2.cpp:28-125):
                  every row once, slot by slot, input order kept within a
                  slot. The slot function is this project's (a mix of the
                  rows' key hash, below); the reference's is Arrow's
                  HashMultiColumn, and which slot a key lands in changes no
                  query result.
  limit_sort    - LimitSortPOp::selectK
                  (fpdb-executor/src/physical/limitsort/LimitSortPOp.cpp:97-135,
                  arrow::compute::SelectKUnstable + Take): the first k rows in
                  key order; ties kept in input order.
"""

from __future__ import annotations

import datetime as _dt

import numpy as np

from flexpushdowndb_gb300.tupleset import Column, Table

from . import expr as _expr

# ------------------------------------------------------------------ filter


def take(table: Table, idx: np.ndarray, names=None) -> Table:
    cols = []
    for c in table.columns:
        if names is not None and c.name not in names:
            continue
        if c.type == "utf8":
            vals = c.to_list()
            cols.append(Column(c.name, c.type, [vals[i] for i in idx]))
        else:
            cols.append(Column(c.name, c.type, c.values[idx]))
    if names is not None:
        order = {n: i for i, n in enumerate(names)}
        cols.sort(key=lambda c: order[c.name])
    return Table(cols)


def filter_table(table: Table, predicate: dict | None, project=None) -> Table:
    mask = np.ones(table.num_rows, dtype=bool) if predicate is None else _expr.predicate(predicate, table)
    idx = np.nonzero(mask)[0]
    names = None if project is None else [n for n in project if n in table.names]
    return take(table, idx, names)


# ------------------------------------------------------------------- bloom

_U = np.uint64


def mix64(k: np.ndarray) -> np.ndarray:
    """MurmurHash3's 64-bit finaliser (Austin Appleby, public domain)."""
    with np.errstate(over="ignore"):
        k = k.astype(np.uint64)
        k ^= k >> _U(33)
        k *= _U(0xFF51AFD7ED558CCD)
        k ^= k >> _U(33)
        k *= _U(0xC4CEB9FE1A85EC53)
        k ^= k >> _U(33)
    return k


def hash_key(v: np.ndarray) -> np.ndarray:
    return mix64(np.asarray(v).astype(np.int64).view(np.uint64) ^ _U(0x9E3779B97F4A7C15))


def hash_bytes(b: bytes) -> int:
    """FNV-1a over the bytes, then the length folded in and mixed."""
    h = 0xCBF29CE484222325
    for x in b:
        h = ((h ^ x) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return int(mix64(np.array([h ^ len(b)], dtype=np.uint64))[0])


def row_key_hash(table: Table, keys) -> np.ndarray:
    """Per-row hash of a key of several columns (integers by value, utf8 by
    bytes), each column folded in with a boost-style combine and a mix."""
    h = np.full(table.num_rows, 0x243F6A8885A308D3, dtype=np.uint64)
    for k in keys:
        c = table.column(k)
        if c.type == "utf8":
            v = np.array([hash_bytes(s.encode()) for s in c.to_list()], dtype=np.uint64)
        else:
            v = hash_key(np.asarray(c.values))
        with np.errstate(over="ignore"):
            h = mix64(h ^ (v + _U(0x9E3779B97F4A7C15) + (h << _U(6)) + (h >> _U(2))))
    return h


def shuffle_slots(table: Table, keys, num_slots: int) -> np.ndarray:
    g = mix64(row_key_hash(table, keys) ^ _U(0x5851F42D4C957F2D))
    return (((g >> _U(32)) * _U(num_slots)) >> _U(32)).astype(np.int64)


def shuffle(table: Table, keys, num_slots: int) -> tuple[Table, list[int]]:
    """The rows slot by slot (stable), and the num_slots + 1 slot offsets."""
    slot = shuffle_slots(table, keys, num_slots)
    order = np.argsort(slot, kind="stable")
    counts = np.bincount(slot, minlength=num_slots)
    return take(table, order), [0] + np.cumsum(counts).tolist()


def bloom_hash(v: np.ndarray) -> np.ndarray:
    """The filter's key hash: a multiply by 2^64 / phi (Fibonacci hashing),
    then the high bits folded into the low ones (h ^ h >> 29)."""
    with np.errstate(over="ignore"):
        h = np.asarray(v).astype(np.int64).view(np.uint64) * _U(0x9E3779B97F4A7C15)
        return h ^ (h >> _U(29))


def bloom_num_blocks(n_keys: int, bits_per_key: int) -> int:
    return max(1, (n_keys * bits_per_key + 255) // 256)


def bloom_words(keys: np.ndarray, bits_per_key: int = 10, num_hashes: int = 3) -> np.ndarray:
    nb = bloom_num_blocks(len(keys), bits_per_key)
    words = np.zeros(nb * 8, dtype=np.uint32)
    h = bloom_hash(keys)
    blk = ((h >> _U(32)) * _U(nb)) >> _U(32)
    for i in range(num_hashes):
        b = (h >> _U(8 * i)) & _U(0xFF)
        w = (blk * _U(8) + (b >> _U(5))).astype(np.int64)
        bit = (np.uint32(1) << (b & _U(31)).astype(np.uint32)).astype(np.uint32)
        np.bitwise_or.at(words, w, bit)
    return words


def bloom_contains(words: np.ndarray, keys: np.ndarray, num_hashes: int = 3) -> np.ndarray:
    nb = len(words) // 8
    h = bloom_hash(keys)
    blk = ((h >> _U(32)) * _U(nb)) >> _U(32)
    ok = np.ones(len(keys), dtype=bool)
    for i in range(num_hashes):
        b = (h >> _U(8 * i)) & _U(0xFF)
        w = words[(blk * _U(8) + (b >> _U(5))).astype(np.int64)]
        ok &= ((w >> (b & _U(31)).astype(np.uint32)) & np.uint32(1)).astype(bool)
    return ok


def bloom_use(table: Table, words: np.ndarray, key: str, num_hashes: int = 3) -> Table:
    return take(table, np.nonzero(bloom_contains(words, table[key], num_hashes))[0])


# -------------------------------------------------------------------- join


def join_indices(build_keys: np.ndarray, probe_keys: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """All (probe_row, build_row) pairs with equal keys."""
    bk = np.asarray(build_keys, dtype=np.int64)
    pk = np.asarray(probe_keys, dtype=np.int64)
    order = np.argsort(bk, kind="stable")
    sk = bk[order]
    lo = np.searchsorted(sk, pk, "left")
    hi = np.searchsorted(sk, pk, "right")
    cnt = hi - lo
    total = int(cnt.sum())
    probe_idx = np.repeat(np.arange(len(pk)), cnt)
    starts = np.repeat(lo, cnt)
    within = np.arange(total) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    build_idx = order[starts + within]
    return probe_idx, build_idx


def hash_join(build: Table, probe: Table, build_key: str, probe_key: str, needed=None) -> Table:
    pi, bi = join_indices(build[build_key], probe[probe_key])
    cols = []
    for t, idx in ((probe, pi), (build, bi)):
        for c in t.columns:
            if needed is not None and c.name not in needed:
                continue
            if c.type == "utf8":
                vals = c.to_list()
                cols.append(Column(c.name, c.type, [vals[i] for i in idx]))
            else:
                cols.append(Column(c.name, c.type, c.values[idx]))
    return Table(cols)


def _take_nullable(t: Table, idx: np.ndarray, names) -> list[Column]:
    """Columns of t at rows idx, a -1 giving a null."""
    out = []
    null = idx < 0
    safe = np.where(null, 0, idx)
    for c in t.columns:
        if names is not None and c.name not in names:
            continue
        if c.type == "utf8":
            vals = c.to_list()
            col = Column(c.name, c.type, ["" if z else vals[i] for i, z in zip(safe.tolist(), null.tolist())])
        else:
            col = Column(c.name, c.type, np.where(null, 0, c.values[safe] if len(c.values) else 0))
        if null.any():
            col.valid = ~null
        out.append(col)
    return out


def hash_join_typed(build: Table, probe: Table, build_key: str, probe_key: str, join_type: str,
                    needed=None) -> Table:
    """The six join types of HashJoinArrowKernel
    (fpdb-executor/src/physical/join/hashjoin/HashJoinArrowKernel.cpp:164-195,
    JoinType.h:13-20; the build side is Arrow's right input): INNER; LEFT
    keeps every build row (Arrow RIGHT_OUTER), RIGHT every probe row
    (LEFT_OUTER), FULL both, the missing side null; LEFT_SEMI the build rows
    with a match (build columns), RIGHT_SEMI the probe rows with a match
    (probe columns). Row order is not part of the result."""
    pi, bi = join_indices(build[build_key], probe[probe_key])
    n_p, n_b = probe.num_rows, build.num_rows
    if join_type == "RIGHT_SEMI":
        rows = np.unique(pi)
        return Table(_take_nullable(probe, rows, needed))
    if join_type == "LEFT_SEMI":
        rows = np.unique(bi)
        return Table(_take_nullable(build, rows, needed))
    pi, bi = list(pi), list(bi)
    if join_type in ("RIGHT", "FULL"):
        hit = np.zeros(n_p, dtype=bool)
        hit[np.asarray(pi, dtype=np.int64)] = True
        for r in np.nonzero(~hit)[0].tolist():
            pi.append(r)
            bi.append(-1)
    if join_type in ("LEFT", "FULL"):
        hit = np.zeros(n_b, dtype=bool)
        hit[np.asarray([b for b in bi if b >= 0], dtype=np.int64)] = True
        for r in np.nonzero(~hit)[0].tolist():
            pi.append(-1)
            bi.append(r)
    elif join_type not in ("INNER", "RIGHT"):
        raise ValueError(join_type)
    pi, bi = np.asarray(pi, dtype=np.int64), np.asarray(bi, dtype=np.int64)
    return Table(_take_nullable(probe, pi, needed) + _take_nullable(build, bi, needed))


# ------------------------------------------------------------------- group


def hash_join_keys(build: Table, probe: Table, build_keys, probe_keys, needed=None) -> Table:
    """Inner join on several key columns (HashJoinPredicate's column lists,
    fpdb-executor/include/fpdb/executor/physical/join/hashjoin/HashJoinPredicate.h:25-26):
    every (probe, build) pair whose key columns are equal pairwise; probe
    columns then build columns."""
    bk = list(zip(*[build[k] if isinstance(build[k], list) else build[k].tolist() for k in build_keys]))
    pk = list(zip(*[probe[k] if isinstance(probe[k], list) else probe[k].tolist() for k in probe_keys]))
    index: dict = {}
    for r, k in enumerate(bk):
        index.setdefault(k, []).append(r)
    pi, bi = [], []
    for r, k in enumerate(pk):
        for b in index.get(k, ()):
            pi.append(r)
            bi.append(b)
    pnames = [n for n in probe.names if needed is None or n in needed]
    bnames = [n for n in build.names if needed is None or n in needed]
    p = take(probe, np.array(pi, dtype=np.int64), pnames if needed is not None else None)
    b = take(build, np.array(bi, dtype=np.int64), bnames if needed is not None else None)
    return Table(p.columns + b.columns)


def group_by(table: Table, group_cols: list[str], aggregates: list[dict]) -> Table:
    """aggregates: [{"function": SUM|COUNT|MIN|MAX|AVG|AVG_REDUCE, "name": .., "expr": ..}]"""
    n = table.num_rows
    keys = [np.array(table[g], dtype=object) if table.column(g).type == "utf8" else table[g] for g in group_cols]
    if n == 0:
        uniq_rows: list[tuple] = []
        inv = np.zeros(0, dtype=np.int64)
    elif not group_cols:
        # a non-grouped aggregate (AggregatePOp): one group of every row
        uniq_rows = [()]
        inv = np.zeros(n, dtype=np.int64)
    else:
        tuples = list(zip(*[k.tolist() for k in keys]))
        index: dict = {}
        inv = np.empty(n, dtype=np.int64)
        for i, t in enumerate(tuples):
            inv[i] = index.setdefault(t, len(index))
        uniq_rows = list(index.keys())
    g = len(uniq_rows)
    cols = []
    for j, name in enumerate(group_cols):
        c = table.column(name)
        vals = [r[j] for r in uniq_rows]
        cols.append(Column(name, c.type, vals if c.type == "utf8" else np.array(vals, dtype=np.int64)))
    for a in aggregates:
        fn = a["function"].upper()
        if fn == "AVG_REDUCE":
            # AvgReduce (fpdb-executor/src/physical/aggregate/function/AvgReduce.cpp:21-84)
            sc, cc = table.column("AVG_INTERMEDIATE_SUM_" + a["name"]), table.column("AVG_INTERMEDIATE_COUNT_" + a["name"])
            is_f = sc.type == "float64"
            s = np.zeros(g, dtype=np.float64 if is_f else np.int64)
            cnt = np.zeros(g, dtype=np.int64)
            with np.errstate(over="ignore"):
                np.add.at(s, inv, sc.values)
                np.add.at(cnt, inv, cc.values)
            cols.append(Column(a["name"], "float64", s.astype(np.float64) / np.maximum(cnt, 1)))
            continue
        if fn == "COUNT":
            cnt = np.bincount(inv, minlength=g).astype(np.int64) if g else np.zeros(0, np.int64)
            cols.append(Column(a["name"], "int64", cnt))
            continue
        v, vt = _expr.value(a["expr"], table)
        v = np.broadcast_to(np.asarray(v), (n,))
        is_f = vt == "float64"
        if fn in ("SUM", "AVG"):
            if is_f:
                s = np.zeros(g, dtype=np.float64)
                np.add.at(s, inv, v.astype(np.float64))
            else:
                s = np.zeros(g, dtype=np.int64)
                with np.errstate(over="ignore"):
                    np.add.at(s, inv, v.astype(np.int64))  # two's-complement wrap, like hash_sum
            if fn == "SUM":
                cols.append(Column(a["name"], "float64" if is_f else "int64", s))
            else:
                cnt = np.bincount(inv, minlength=g)
                cols.append(Column(a["name"], "float64", s.astype(np.float64) / np.maximum(cnt, 1)))
        elif fn in ("MIN", "MAX"):
            init = np.inf if is_f else (np.iinfo(np.int64).max if fn == "MIN" else np.iinfo(np.int64).min)
            if fn == "MAX" and is_f:
                init = -np.inf
            s = np.full(g, init, dtype=np.float64 if is_f else np.int64)
            (np.minimum if fn == "MIN" else np.maximum).at(s, inv, v.astype(s.dtype))
            cols.append(Column(a["name"], vt, s))
        else:
            raise _expr.OracleError(f"aggregate {fn}")
    return Table(cols)


# --------------------------------------------------------------------- CSV


def days_from_civil(y: int, m: int, d: int) -> int:
    return (_dt.date(y, m, d) - _dt.date(1970, 1, 1)).days


def csv_parse(text: bytes, fields: list[tuple[str, str]], columns=None, delimiter: str = ",",
              has_header: bool = False) -> Table:
    lines = text.split(b"\n")
    if lines and lines[-1] == b"":
        lines = lines[:-1]
    if has_header and lines:
        lines = lines[1:]
    rows = []
    for ln in lines:
        if ln.endswith(b"\r"):
            ln = ln[:-1]
        parts = ln.split(delimiter.encode())
        if len(parts) != len(fields):
            raise _expr.OracleError("wrong field count")
        rows.append([p[1:-1] if len(p) >= 2 and p[:1] == b'"' and p[-1:] == b'"' else p for p in parts])
    want = [n for n, _ in fields] if columns is None else list(columns)
    out = []
    for name in want:
        k = [n for n, _ in fields].index(name)
        ty = fields[k][1]
        raw = [r[k] for r in rows]
        if ty == "utf8":
            out.append(Column(name, "utf8", [x.decode() for x in raw]))
        elif ty == "date32":
            out.append(Column(name, "date32",
                              [days_from_civil(int(x[:4]), int(x[5:7]), int(x[8:10])) for x in raw]))
        elif ty.startswith("decimal"):
            scale = int(ty[ty.index(",") + 1 : ty.index(")")])
            vals = []
            for x in raw:
                s = x.decode()
                neg = s.startswith("-")
                s = s.lstrip("+-")
                ip, _, fp = s.partition(".")
                if len(fp) > scale:
                    raise _expr.OracleError("too many fractional digits")
                v = int(ip or "0") * 10**scale + int((fp + "0" * scale)[:scale] or "0")
                vals.append(-v if neg else v)
            out.append(Column(name, "int64", vals))
        else:
            out.append(Column(name, ty, [int(x) for x in raw]))
    return Table(out)


# ----------------------------------------------------------- project / sort


def project(table: Table, exprs=(), pairs=()) -> Table:
    cols = []
    for a, b in pairs:
        c = table.column(a)
        cols.append(Column(b, c.type, c.values))
    for name, e in exprs:
        v, ty = _expr.value(e, table)
        cols.append(Column(name, ty, v))
    return Table(cols)


def limit_sort(table: Table, k: int, sort_keys) -> Table:
    """sort_keys: (column, "ASC" | "DESC") pairs."""
    import functools

    cols = {n: table[n] for n, _ in sort_keys}

    def cmp(a, b):
        for n, order in sort_keys:
            x, y = cols[n][a], cols[n][b]
            if isinstance(x, str):
                x, y = x.encode(), y.encode()
            r = int(x > y) - int(x < y)
            if r:
                return -r if order == "DESC" else r
        return (a > b) - (a < b)

    idx = sorted(range(table.num_rows), key=functools.cmp_to_key(cmp))[:k]
    return take(table, np.array(idx, dtype=np.int64))
