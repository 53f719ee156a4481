"""The request server: every request's result is the same served alone and
in a concurrent mix (batched star queries, overlapping plans on several
workers, a column cache that evicts, admission that waits), and equal to
the oracle's."""

import json

import pytest

from flexpushdowndb_gb300 import GfpdbError, serving, workloads
from flexpushdowndb_gb300.tupleset import text_table
from oracle import queries
from oracle import ops as oops
from flexpushdowndb_gb300.expression import col, lt, num_lit

pytestmark = pytest.mark.gpu


def small_world(seed=6000):
    """Tables of every serving template, small enough for the oracle."""
    sizes = workloads.batch_partition_sizes(4, lo=2_000, hi=60_000, seed=seed)
    tabs = workloads.batch_tables(4, sizes=sizes, seed=seed)
    parts = [f"p{i}" for i in range(4)]
    two = workloads.two_table_tables(fact_rows=120_000, seed=seed + 1)
    star = workloads.star_tables(fact_rows=150_000, seed=seed + 2)
    tables = dict(tabs)
    tables["fact"], tables["dim"] = two["fact"], two["dim"]
    tables["sfact"] = star["fact"]
    for i in range(1, 5):
        tables[f"s{i}"] = star[f"d{i}"]
    tables["g"] = workloads.groupby_table(100_000, 50_000, seed=seed + 3)
    csv_text = workloads.lineitem_csv(8_000, seed=seed + 4)
    tables["lineitem"] = text_table(csv_text)
    return tables, parts, two, star, csv_text


def star_plan_on(prefix_fact="sfact", dim_prefix="s", consts=(1, 3, 2, 5)):
    d = json.loads(workloads.star_plan(consts=consts).to_json())
    for o in d["ops"]:
        if o["type"] == "TableScanPOp":
            o["table"] = prefix_fact if o["table"] == "fact" else dim_prefix + o["table"][1:]
    return d


def requests_and_answers(tables, parts, two, star, csv_text, n_star=24):
    template = serving.star_batch_template(workloads.star_batch_spec(parts, []))
    qs = workloads.batch_queries(n_star, seed=6100)
    reqs, want = [], []
    for k, q in enumerate(qs):
        reqs.append({"kind": "star", "batch": template, "ranges": [list(r) for r in q]})
        want.append(queries.star_query_ranges(tables, parts, q).sorted_rows())
        if k % 6 == 0:
            reqs.append({"kind": "plan", "plan": json.loads(workloads.two_table_plan().to_json())})
            want.append(queries.two_table_query(two).sorted_rows())
        if k % 8 == 1:
            consts = (k % 5, k % 25, k % 7, k % 7)
            reqs.append({"kind": "plan", "plan": star_plan_on(consts=consts)})
            want.append(queries.star_query(star, consts=consts).sorted_rows())
        if k % 12 == 2:
            p = json.loads(workloads.groupby_plan().to_json())
            p["ops"][0]["table"] = "g"
            reqs.append({"kind": "plan", "plan": p})
            want.append(oops.group_by(tables["g"], ["k"], [{"function": "SUM", "name": "s", "expr": col("v")},
                                                           {"function": "COUNT", "name": "c"}]).sorted_rows())
        if k % 12 == 5:
            reqs.append({"kind": "plan", "plan": json.loads(workloads.csv_scan_plan().to_json())})
            t = oops.csv_parse(csv_text, workloads.LINEITEM_FIELDS, delimiter="|")
            sel = oops.filter_table(t, workloads.csv_scan_predicate())
            s = sum(int(a) * int(b) for a, b in zip(sel["d2"], sel["i2"]))
            want.append([(s, sel.num_rows)] if sel.num_rows else [])
    return reqs, want


@pytest.fixture(scope="module")
def world():
    return small_world()


def served(server, tables, reqs):
    for name, t in tables.items():
        server.register(name, t)
    tickets = [server.submit(r) for r in reqs]
    out = []
    for t in tickets:
        res, st = server.wait(t)
        out.append((res.sorted_rows(), st))
    return out


def test_mixed_requests_match_alone_and_oracle(gpu, world):
    tables, parts, two, star, csv_text = world
    reqs, want = requests_and_answers(tables, parts, two, star, csv_text)
    with serving.Server(workers=3, cache_bytes=8 << 30, hbm_budget_bytes=16 << 30) as mixed:
        got_mix = served(mixed, tables, reqs)
        stats = mixed.stats()
    with serving.Server(workers=1, batching=False, cuda_graphs=False, cache_bytes=8 << 30,
                        hbm_budget_bytes=16 << 30) as alone:
        got_alone = served(alone, tables, reqs)
    for i, (w, (m, sm), (a, sa)) in enumerate(zip(want, got_mix, got_alone)):
        assert m == a, f"request {i}: mix differs from alone"
        assert m == w, f"request {i}: differs from the oracle"
        assert sa["batch_size"] == 1
    assert max(s["batch_size"] for _, s in got_mix) > 1, "no star requests were batched"
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["batches"] >= 1 and stats["cache_hits"] > 0


def test_small_cache_evicts_and_stays_exact(gpu, world):
    tables, parts, two, star, csv_text = world
    reqs, want = requests_and_answers(tables, parts, two, star, csv_text, n_star=12)
    # room for a few columns at a time: every template reloads what it needs
    with serving.Server(workers=2, cache_bytes=12 << 20, hbm_budget_bytes=4 << 30) as sv:
        got = served(sv, {k: v for k, v in tables.items() if k != "lineitem"},
                      [r for r in reqs if "CsvScanPOp" not in json.dumps(r)])
        st = sv.stats()
    w = [x for r, x in zip(reqs, want) if "CsvScanPOp" not in json.dumps(r)]
    assert [g for g, _ in got] == w
    assert st["cache_evictions"] > 0
    assert st["cache_bytes"] <= 12 << 20


def test_admission_waits_within_budget(gpu, world):
    tables, parts, two, star, csv_text = world
    plan = json.loads(workloads.two_table_plan().to_json())
    # the working budget (hbm budget - cache) admits one plan at a time
    with serving.Server(workers=4, cache_bytes=1 << 30, hbm_budget_bytes=(1 << 30) + (80 << 20)) as sv:
        sv.register("fact", tables["fact"])
        sv.register("dim", tables["dim"])
        tickets = [sv.submit({"kind": "plan", "plan": plan}) for _ in range(8)]
        res = [sv.wait(t)[0].sorted_rows() for t in tickets]
        st = sv.stats()
    assert all(r == queries.two_table_query(two).sorted_rows() for r in res)
    assert st["admission_waits"] > 0


def test_errors_are_per_request(gpu, world):
    tables, parts, two, star, csv_text = world
    with serving.Server(workers=2) as sv:
        sv.register("fact", tables["fact"])
        sv.register("dim", tables["dim"])
        with pytest.raises(GfpdbError):
            sv.submit({"kind": "plan", "plan": star_plan_on()})  # tables not registered
        bad = json.loads(workloads.two_table_plan().to_json())
        for o in bad["ops"]:
            if o["type"] == "FilterPOp":
                o["predicate"] = lt(col("nope"), num_lit(1))
        t_bad = sv.submit({"kind": "plan", "plan": bad})
        t_ok = sv.submit({"kind": "plan", "plan": json.loads(workloads.two_table_plan().to_json())})
        with pytest.raises(GfpdbError):
            sv.wait(t_bad)
        assert sv.wait(t_ok)[0].sorted_rows() == queries.two_table_query(two).sorted_rows()
        with pytest.raises(GfpdbError):
            sv.wait(t_bad)  # a ticket is collected once
        assert sv.stats()["failed"] == 1
