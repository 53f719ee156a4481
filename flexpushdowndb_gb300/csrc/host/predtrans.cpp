// Predicate transfer planning: the bloom-filter operators a join graph gets,
// in the order SmallToLargePredTransOrder builds them
// (fpdb-executor/src/physical/transform/pred-trans/SmallToLargePredTransOrder.cpp:14-214).
//
// Input: the base tables (the operator that produces each one, with its row
// count) and the joins between them (JoinOriginTracer's join origins,
// fpdb-plan/src/prephysical/JoinOriginTracer.cpp:199-240). Each join is
// oriented from its smaller to its larger table (the join type reversed when
// the sides swap), joins between the same two tables with the same type
// merge, and FULL joins transfer nothing. A join then gets
//   - a forward filter (unless RIGHT): created on the smaller table's key,
//     used on the larger table's;
//   - a backward filter (unless LEFT): created on the larger table's key,
//     used on the smaller table's.
// Forward filters are placed in topological order: a table's filter is
// created only after every forward filter aimed at that table has been
// applied to it, so selections travel from small tables to large ones
// transitively; each use becomes the table's new output. Backward filters
// follow, from the tables that receive no backward filter (the largest)
// down. A cycle in either direction is an error. Every table's last operator
// is where its joins attach.
//
// The reference visits ready filters in hash-set order; here they go in
// order of the smaller table's selectivity (the fraction of its rows its
// local filters keep, a hint that defaults to 1: the most selective filter
// is applied to the larger table first), then its rows, then the larger
// table's rows, then input order, so a plan is reproducible. A join on
// several column pairs transfers a filter on its first pair (a filter on
// part of the key still drops no matching row).
#include <algorithm>
#include <map>
#include <queue>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "pop.h"

namespace gfpdb::pop {

namespace {

std::string quote(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
  }
  return o + "\"";
}

struct Edge {
  std::string left, right;  // smaller, larger table
  std::vector<std::string> lcols, rcols;
  JoinKind kind;
  int64_t lrows, rrows;
  double lsel;
  size_t order;  // input position
};

JoinKind reversed(JoinKind k) {  // reverseJoinType (fpdb-plan/include/fpdb/plan/prephysical/JoinType.h:22-40)
  switch (k) {
    case JoinKind::Left: return JoinKind::Right;
    case JoinKind::Right: return JoinKind::Left;
    case JoinKind::LeftSemi: return JoinKind::RightSemi;
    case JoinKind::RightSemi: return JoinKind::LeftSemi;
    default: return k;
  }
}

struct Node {
  std::string create, use;  // operator names
  std::string create_col, use_col;
  std::string create_unit, use_unit;  // tables
};

}  // namespace

std::string plan_predicate_transfer(const json::Value& spec) {
  std::map<std::string, int64_t> rows;
  std::map<std::string, double> sel;
  std::vector<std::string> tables;
  for (auto& t : spec.at("tables").array()) {
    const std::string op = t.at("op").str();
    if (rows.count(op)) fail(GFPDB_EINVAL, "predicate transfer: table '" + op + "' listed twice");
    rows[op] = t.get_int("rowCount", 0);
    sel[op] = t.get_num("selectivity", 1.0);
    tables.push_back(op);
  }
  const int bits = static_cast<int>(spec.get_int("bitsPerKey", 10));
  const int hashes = static_cast<int>(spec.get_int("numHashes", 3));
  const std::string prefix = spec.get_str("namePrefix", "pt");

  // join origins, oriented small -> large and merged
  std::vector<Edge> edges;
  size_t order = 0;
  for (auto& j : spec.at("joins").array()) {
    Edge e;
    e.left = j.at("left").str();
    e.right = j.at("right").str();
    e.lcols = j.str_list("leftColumns");
    e.rcols = j.str_list("rightColumns");
    e.kind = join_kind_from_name(j.get_str("joinType", "INNER"));
    if (!rows.count(e.left) || !rows.count(e.right))
      fail(GFPDB_EINVAL, "predicate transfer: a join names a table that is not listed");
    if (e.left == e.right) fail(GFPDB_EINVAL, "predicate transfer: a join of a table with itself");
    if (e.lcols.empty() || e.lcols.size() != e.rcols.size())
      fail(GFPDB_EINVAL, "predicate transfer: a join needs as many left as right columns, at least one");
    if (rows[e.left] > rows[e.right]) {
      std::swap(e.left, e.right);
      std::swap(e.lcols, e.rcols);
      e.kind = reversed(e.kind);
    }
    e.lrows = rows[e.left];
    e.rrows = rows[e.right];
    e.lsel = sel[e.left];
    e.order = order++;
    bool merged = false;
    for (auto& x : edges)
      if (x.left == e.left && x.right == e.right && x.kind == e.kind) {
        x.lcols.insert(x.lcols.end(), e.lcols.begin(), e.lcols.end());
        x.rcols.insert(x.rcols.end(), e.rcols.begin(), e.rcols.end());
        merged = true;
        break;
      }
    if (!merged) edges.push_back(std::move(e));
  }
  std::stable_sort(edges.begin(), edges.end(), [](const Edge& a, const Edge& b) {
    if (a.lsel != b.lsel) return a.lsel < b.lsel;
    if (a.lrows != b.lrows) return a.lrows < b.lrows;
    if (a.rrows != b.rrows) return a.rrows < b.rrows;
    return a.order < b.order;
  });

  // filter operators and the two transfer graphs
  std::vector<Node> fw, bw;
  std::map<std::string, int> fw_to_visit, bw_to_visit;
  std::map<std::string, std::vector<size_t>> fw_out, bw_out;
  for (size_t k = 0; k < edges.size(); ++k) {
    const Edge& e = edges[k];
    if (e.kind == JoinKind::Full) continue;  // no transfer across FULL joins
    if (e.kind != JoinKind::Right) {
      Node n{prefix + "_bf_create_fw" + std::to_string(k), prefix + "_bf_use_fw" + std::to_string(k), e.lcols[0],
             e.rcols[0], e.left, e.right};
      fw_out[e.left].push_back(fw.size());
      ++fw_to_visit[e.right];
      fw.push_back(n);
    }
    if (e.kind != JoinKind::Left) {
      Node n{prefix + "_bf_create_bw" + std::to_string(k), prefix + "_bf_use_bw" + std::to_string(k), e.rcols[0],
             e.lcols[0], e.right, e.left};
      bw_out[e.right].push_back(bw.size());
      ++bw_to_visit[e.left];
      bw.push_back(n);
    }
  }

  std::map<std::string, std::string> cur;  // each table's current output operator
  for (auto& t : tables) cur[t] = t;
  std::ostringstream ops, conn;
  bool first_op = true, first_edge = true;
  auto edge = [&](const std::string& p, const std::string& c) {
    conn << (first_edge ? "" : ",") << "[" << quote(p) << "," << quote(c) << "]";
    first_edge = false;
  };
  auto place = [&](std::vector<Node>& nodes, std::map<std::string, int>& to_visit,
                   std::map<std::string, std::vector<size_t>>& out, const char* dir) {
    std::map<std::string, int> visited;
    std::vector<bool> done(nodes.size(), false);
    std::queue<size_t> ready;
    for (size_t i = 0; i < nodes.size(); ++i)
      if (to_visit[nodes[i].create_unit] == 0) ready.push(i);
    size_t placed = 0;
    while (!ready.empty()) {
      const size_t i = ready.front();
      ready.pop();
      if (done[i]) continue;
      done[i] = true;
      ++placed;
      const Node& n = nodes[i];
      ops << (first_op ? "" : ",") << "{\"type\":\"BloomFilterCreatePOp\",\"name\":" << quote(n.create)
          << ",\"bloomFilterColumn\":" << quote(n.create_col) << ",\"bitsPerKey\":" << bits
          << ",\"numHashes\":" << hashes << ",\"bloomFilterUsePOps\":[" << quote(n.use) << "]}";
      ops << ",{\"type\":\"BloomFilterUsePOp\",\"name\":" << quote(n.use) << ",\"bloomFilterColumn\":"
          << quote(n.use_col) << "}";
      first_op = false;
      edge(cur[n.create_unit], n.create);
      edge(n.create, n.use);
      edge(cur[n.use_unit], n.use);
      cur[n.use_unit] = n.use;
      if (++visited[n.use_unit] == to_visit[n.use_unit])
        for (size_t o : out[n.use_unit]) ready.push(o);
    }
    if (placed != nodes.size())
      fail(GFPDB_EINVAL, std::string("predicate transfer: the joins contain a cycle (") + dir + " transfer)");
  };
  place(fw, fw_to_visit, fw_out, "forward");
  place(bw, bw_to_visit, bw_out, "backward");

  std::ostringstream res;
  res << "{\"ops\":[" << ops.str() << "],\"edges\":[" << conn.str() << "],\"outputs\":{";
  bool first = true;
  for (auto& t : tables) {
    res << (first ? "" : ",") << quote(t) << ":" << quote(cur[t]);
    first = false;
  }
  res << "}}";
  return res.str();
}

}  // namespace gfpdb::pop
