"""The multi-rank path on CPU: two gloo ranks, each computing the star
query over its own fact partitions (with the oracle, standing in for its
GPU), merge their partial group tables; the merge equals the query over all
partitions. Also the merge alone, with int64 wrap-around."""

import os
import socket

import pytest

from flexpushdowndb_gb300 import distributed, workloads
from flexpushdowndb_gb300.tupleset import Column, Table


def test_merge_partials_wraps_and_groups():
    a = Table([Column("g", "int32", [1, 2]), Column("s", "int64", [2**62, 5]), Column("c", "int64", [1, 1])])
    b = Table([Column("g", "int32", [2, 1]), Column("s", "int64", [7, 2**62]), Column("c", "int64", [2, 3])])
    m = distributed.merge_partials([a, b, Table([])], ["g"], ["s", "c"])
    got = dict((r[0], r[1:]) for r in m.rows())
    assert got[1] == (-(2**63), 4)  # 2^62 + 2^62 wraps to -2^63
    assert got[2] == (12, 3)


def test_rank_partitions_cover_all():
    parts = [distributed.rank_partitions(10, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == list(range(10))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    from oracle import queries

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = workloads.batch_partition_sizes(6, lo=2_000, hi=40_000, seed=9100)
    tabs = workloads.batch_tables(6, sizes=sizes, seed=9100)
    ranges = [(0, 39), (0, 24), (3, 50), (0, 99)]
    mine = [f"p{i}" for i in distributed.rank_partitions(6, rank, world)]
    partial = queries.star_query_ranges(tabs, mine, ranges)
    merged = distributed.gather_and_merge(partial, ["d2_g", "d4_g"], ["revenue", "discount_revenue", "cnt"])
    if rank == 0:
        want = queries.star_query_ranges(tabs, [f"p{i}" for i in range(6)], ranges)
        with open(out_path, "w") as f:
            f.write("ok" if merged.sorted_rows() == want.sorted_rows() else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_pack_table_roundtrip():
    t = Table([Column("a", "int32", [1, -2, 3]), Column("s", "utf8", ["", "xy", "zzz"]),
               Column("f", "float64", [0.5, 1.5, -2.0]), Column("d", "date32", [1, 2, 3])])
    u = distributed.unpack_table(distributed.pack_table(t))
    assert u.names == t.names and u.rows() == t.rows()
    assert [c.type for c in u.columns] == [c.type for c in t.columns]
    assert distributed.unpack_table(distributed.pack_table(Table([Column("a", "int64", [])]))).num_rows == 0


def _exchange_main(rank, world, port, out_path):
    """Each rank: a partial group-by of its shard (oracle), the partitioned
    exchange (oracle shuffle standing in for the device one), the reduce
    (oracle group-by with the reduce functions)."""
    import numpy as np
    import torch.distributed as dist

    from flexpushdowndb_gb300 import plan
    from flexpushdowndb_gb300.expression import col
    from oracle import ops as oops

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n = 60_000
    keys = workloads.zipf_keys(n, 20_000, seed=77)
    vals = np.random.default_rng(77).integers(-(2**40), 2**40, n)
    whole = Table([Column("k", "int64", keys), Column("v", "int64", vals)])
    aggs = [{"function": "SUM", "name": "s", "expr": col("v")}, {"function": "COUNT", "name": "c"},
            {"function": "MIN", "name": "lo", "expr": col("v")}, {"function": "AVG", "name": "avg", "expr": col("v")}]
    mine = Table([Column("k", "int64", keys[rank::world]), Column("v", "int64", vals[rank::world])])
    partial = oops.group_by(mine, ["k"], plan.partial_aggregates(aggs))

    def shuffle(t, ks, slots):
        rows, offs = oops.shuffle(t, ks, slots)
        return [rows.slice(offs[i], offs[i + 1]) for i in range(slots)]

    def reduce(parts, ks, raggs):
        return oops.group_by(Table.concat(parts), ks, raggs)

    share = distributed.exchange_and_reduce(partial, ["k"], aggs, shuffle=shuffle, reduce=reduce)
    shares = [None] * world
    dist.all_gather_object(shares, share.rows())
    if rank == 0:
        want = oops.group_by(whole, ["k"], aggs).sorted_rows()
        got = sorted(sum(shares, []))
        key_sets = [set(r[0] for r in s) for s in shares]
        disjoint = all(not (key_sets[i] & key_sets[j]) for i in range(world) for j in range(i + 1, world))
        with open(out_path, "w") as f:
            f.write("ok" if got == want and disjoint and all(shares) else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_partitioned_exchange(tmp_path):
    torch_mp = pytest.importorskip("torch.multiprocessing")
    out = tmp_path / "result.txt"
    torch_mp.spawn(_exchange_main, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    assert out.read_text() == "ok"


def test_two_gloo_ranks_merge_star_partials(tmp_path):
    torch_mp = pytest.importorskip("torch.multiprocessing")
    out = tmp_path / "result.txt"
    torch_mp.spawn(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    assert out.read_text() == "ok"
