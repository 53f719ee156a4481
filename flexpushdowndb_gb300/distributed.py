"""Multi-GPU form: one process per GPU, each over its own fact partitions.

The fact table shards by partition with no exchange on the data path; the
one exchange is the merge of every rank's partial group table, the
reference's two-phase group-by
(fpdb-executor/src/physical/transform/PrePToPTransformer.cpp:434-580):

  exchange_and_reduce  each rank hash-partitions its partial table on the
                       group columns into one slot per rank (the device
                       shuffle, gfpdb_shuffle, as ShuffleKernel2::shuffle
                       feeds the reduce ops), the slots travel rank to rank
                       in one all-to-all, and each rank reduces what it
                       received with the device group-by (SUM of partial sums
                       and counts, MIN / MAX of partial minima / maxima,
                       AVG_REDUCE), ending with a disjoint share of the
                       groups: the high-cardinality path (10M-key group-bys);
  gather_and_merge     every partial table to rank 0, merged there: for
                       results of a few hundred groups (the star query's).

Sums and counts are additive and int64 addition is associative (two's-
complement wrap-around, as Arrow's hash_sum), so either merge is exact in any
rank order.
"""

from __future__ import annotations

import json
from typing import Callable, Sequence

import numpy as np

from .tupleset import Column, Table

# ------------------------------------------------------------ wire format


def pack_table(t: Table) -> np.ndarray:
    """A Table as bytes: an 8-byte header length, a JSON header (names,
    types, rows, buffer sizes), then each column's buffers."""
    bufs, meta = [], []
    for c in t.columns:
        if c.type == "utf8":
            off, data = c.values
            parts = [np.ascontiguousarray(off, dtype=np.int32), np.ascontiguousarray(data, dtype=np.uint8)]
        else:
            parts = [np.ascontiguousarray(c.values)]
        meta.append({"name": c.name, "type": c.type, "sizes": [p.nbytes for p in parts]})
        bufs += parts
    head = json.dumps({"rows": t.num_rows, "columns": meta}).encode()
    total = 8 + len(head) + sum(b.nbytes for b in bufs)
    out = np.empty(total, dtype=np.uint8)
    out[:8] = np.frombuffer(np.int64(len(head)).tobytes(), dtype=np.uint8)
    out[8 : 8 + len(head)] = np.frombuffer(head, dtype=np.uint8)
    at = 8 + len(head)
    for b in bufs:
        out[at : at + b.nbytes] = b.view(np.uint8).reshape(-1)
        at += b.nbytes
    return out


def unpack_table(buf: np.ndarray) -> Table:
    n_head = int(np.frombuffer(buf[:8].tobytes(), dtype=np.int64)[0])
    head = json.loads(buf[8 : 8 + n_head].tobytes())
    at = 8 + n_head
    cols = []
    from .tupleset import NP_TYPES

    for m in head["columns"]:
        sizes = m["sizes"]
        if m["type"] == "utf8":
            off = np.frombuffer(buf[at : at + sizes[0]].tobytes(), dtype=np.int32)
            data = buf[at + sizes[0] : at + sizes[0] + sizes[1]].copy()
            cols.append(Column(m["name"], "utf8", (off, data)))
        else:
            cols.append(Column(m["name"], m["type"], np.frombuffer(buf[at : at + sizes[0]].tobytes(),
                                                                   dtype=NP_TYPES[m["type"]])))
        at += sum(sizes)
    return Table(cols)


# ---------------------------------------------------------------- exchange


def exchange(parts: Sequence[Table], group=None) -> list[Table]:
    """Send parts[r] to rank r; return the part every rank sent here, by
    rank. One all-to-all of the sizes, one of the bytes (CPU tensors under
    gloo, device tensors under NCCL)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    if len(parts) != world:
        raise ValueError(f"exchange needs one part per rank ({world}), got {len(parts)}")
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else None
    packed = [pack_table(p) for p in parts]
    send_sizes = torch.tensor([p.nbytes for p in packed], dtype=torch.int64, device=dev)
    recv_sizes = torch.empty(world, dtype=torch.int64, device=dev)
    dist.all_to_all_single(recv_sizes, send_sizes, group=group)
    send = torch.from_numpy(np.concatenate(packed)).to(dev) if dev is not None else torch.from_numpy(np.concatenate(packed))
    rs = recv_sizes.cpu().tolist()
    recv = torch.empty(int(sum(rs)), dtype=torch.uint8, device=dev)
    dist.all_to_all_single(recv, send, output_split_sizes=rs, input_split_sizes=send_sizes.cpu().tolist(),
                           group=group)
    flat = recv.cpu().numpy()
    out, at = [], 0
    for size in rs:
        out.append(unpack_table(flat[at : at + size]))
        at += size
    return out


def _device_shuffle(t: Table, keys: Sequence[str], slots: int) -> list[Table]:
    from . import ops

    return ops.shuffle_split(t, list(keys), slots)


def _device_reduce(parts: Sequence[Table], keys: Sequence[str], aggregates: Sequence[dict]) -> Table:
    from . import ops

    g = ops.Group(list(keys), list(aggregates))
    for p in parts:
        if p.num_rows:
            g.group(p)
    return g.finalise()


def exchange_and_reduce(partial: Table, key_cols: Sequence[str], aggregates: Sequence[dict], group=None,
                        shuffle: Callable | None = None, reduce: Callable | None = None) -> Table:
    """The second phase of a parallel group-by across ranks. `partial` holds
    this rank's groups with the partial columns of `aggregates` (the
    original aggregate list: plan.partial_aggregates names the columns);
    returns this rank's share of the final groups. `shuffle(table, keys,
    slots)` and `reduce(parts, keys, reduce_aggregates)` default to the
    device shuffle and group-by."""
    import torch.distributed as dist

    from .plan import reduce_aggregates

    world = dist.get_world_size(group)
    parts = (shuffle or _device_shuffle)(partial, key_cols, world)
    received = exchange(parts, group)
    return (reduce or _device_reduce)(received, key_cols, reduce_aggregates(aggregates))


# ------------------------------------------------------- small-result merge


def merge_partials(parts: list[Table], key_cols: list[str], sum_cols: list[str]) -> Table:
    """Group the rows of every partial table by `key_cols` and add up
    `sum_cols` (sums and counts) with int64 wrap-around."""
    parts = [p for p in parts if p.num_rows > 0]
    if not parts:
        return Table([])
    names = parts[0].names
    types = {c.name: c.type for c in parts[0].columns}
    keys = [tuple(r[names.index(k)] for k in key_cols) for p in parts for r in p.rows()]
    vals = {c: np.concatenate([np.asarray(p[c], dtype=np.int64) for p in parts]) for c in sum_cols}
    index: dict = {}
    inv = np.empty(len(keys), dtype=np.int64)
    for i, k in enumerate(keys):
        inv[i] = index.setdefault(k, len(index))
    uniq = list(index)
    cols = []
    for j, k in enumerate(key_cols):
        vs = [u[j] for u in uniq]
        cols.append(Column(k, types[k], vs if types[k] == "utf8" else np.array(vs, dtype=np.int64)))
    for c in sum_cols:
        acc = np.zeros(len(uniq), dtype=np.int64)
        with np.errstate(over="ignore"):
            np.add.at(acc, inv, vals[c])
        cols.append(Column(c, "int64", acc))
    order = key_cols + sum_cols
    return Table([next(c for c in cols if c.name == n) for n in order if n in names])


def gather_and_merge(partial: Table, key_cols: list[str], sum_cols: list[str], group=None) -> Table | None:
    """All ranks contribute their partial table; rank 0 returns the merge,
    the other ranks None."""
    import torch.distributed as dist

    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, partial, group=group)
    return merge_partials(parts, key_cols, sum_cols) if dist.get_rank(group) == 0 else None


def rank_partitions(n_parts: int, rank: int, world: int) -> list[int]:
    """Partition indexes of one rank (round robin)."""
    return list(range(rank, n_parts, world))
