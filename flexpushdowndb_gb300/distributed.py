"""Multi-GPU form: one process per GPU, each over its own fact partitions.

The fact table shards by partition with no exchange on the data path; the
only exchange is the final merge of every rank's partial group table (the
reference's two-phase group-by merges partial aggregates the same way,
fpdb-executor/src/physical/transform/PrePToPTransformer.cpp:434-580). Sums and
counts are additive and int64 addition is associative (two's-complement
wrap-around, as Arrow's hash_sum), so the merge is exact in any rank order.
The partial tables are small (one row per group), so they travel through
torch.distributed's object collectives and are merged on the host.
"""

from __future__ import annotations

import numpy as np

from .tupleset import Column, Table


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
