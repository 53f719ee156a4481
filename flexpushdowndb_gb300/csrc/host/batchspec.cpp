#include "batchspec.h"

#include <cstdio>

namespace gfpdb {

void parse_star_batch_spec(const json::Value& spec, StarBatchSpec& sp) {
  sp.fact_tables = spec.str_list("factTables");
  for (auto& d : spec.at("dimensions").array())
    sp.dims.push_back(
        StarBatchSpec::Dim{d.at("table").str(), d.at("key").str(), d.at("factKey").str(), d.at("filterColumn").str()});
  if (spec.contains("groupBy"))
    for (auto& g : spec.at("groupBy").array())
      sp.group.push_back(StarBatchSpec::Group{static_cast<int>(g.at("dimension").integer()), g.at("column").str()});
  for (auto& a : spec.at("aggregates").array()) {
    StarBatchSpec::Agg agg;
    const std::string f = a.at("function").str();
    if (f == "SUM") agg.fn = AGG_SUM;
    else if (f == "COUNT") agg.fn = AGG_COUNT_STAR;
    else fail(GFPDB_EUNSUPPORTED, "batched star aggregates are SUM and COUNT(*)");
    agg.name = a.at("name").str();
    agg.columns = a.str_list("columns");
    sp.aggs.push_back(agg);
  }
  if (spec.contains("queries"))
    for (auto& q : spec.at("queries").array()) {
      std::vector<std::pair<int64_t, int64_t>> ranges;
      for (auto& r : q.array()) ranges.emplace_back(r.array().at(0).integer(), r.array().at(1).integer());
      if (ranges.size() != sp.dims.size()) fail(GFPDB_EINVAL, "each batched query needs one range per dimension");
      sp.queries.push_back(ranges);
    }
  if (spec.contains("probeOrder"))
    for (auto& o : spec.at("probeOrder").array()) sp.probe_order.push_back(static_cast<int>(o.integer()));
  sp.load_factor = spec.get_num("loadFactor", 0.5);
  if (!(sp.load_factor > 0 && sp.load_factor <= 0.9)) fail(GFPDB_EINVAL, "loadFactor must be in (0, 0.9]");
  sp.items_per_thread = static_cast<int>(spec.get_int("itemsPerThread", 2));
  sp.blocks_per_sm = static_cast<int>(spec.get_int("blocksPerSm", 4));
  sp.stages = static_cast<int>(spec.get_int("stages", 3));
  if (sp.stages < 2 || sp.stages > 8) fail(GFPDB_EINVAL, "stages must be in [2, 8]");
  sp.direct = spec.get_bool("direct", true);
  if (sp.blocks_per_sm < 1 || sp.blocks_per_sm > 16) fail(GFPDB_EINVAL, "blocksPerSm must be in [1, 16]");
  sp.groups_hint = spec.get_int("groupsHint", 1024);
}

std::vector<std::pair<std::string, std::string>> star_batch_columns(const StarBatchSpec& sp) {
  std::vector<std::pair<std::string, std::string>> out;
  auto add = [&](const std::string& t, const std::string& c) {
    for (auto& e : out)
      if (e.first == t && e.second == c) return;
    out.emplace_back(t, c);
  };
  for (auto& t : sp.fact_tables) {
    for (auto& d : sp.dims) add(t, d.fact_key);
    for (auto& a : sp.aggs)
      for (auto& c : a.columns) add(t, c);
  }
  for (size_t d = 0; d < sp.dims.size(); ++d) {
    add(sp.dims[d].table, sp.dims[d].key);
    add(sp.dims[d].table, sp.dims[d].filter);
    for (auto& g : sp.group)
      if (g.dim == static_cast<int>(d)) add(sp.dims[d].table, g.column);
  }
  return out;
}

cudaGraphExec_t capture_star_batch(StarBatch& b, uint64_t* kernels) {
  // run() only clears preallocated buffers and launches kernels: capture it.
  cudaStream_t cs = nullptr;
  GF_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  const uint64_t k0 = g_kernel_launches.load();
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ok = true;
  GF_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  try {
    b.run(cs);
  } catch (const std::exception&) {
    ok = false;
  }
  if (cudaStreamEndCapture(cs, &graph) != cudaSuccess) ok = false;
  if (ok && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) ok = false;
  if (graph) (void)cudaGraphDestroy(graph);
  (void)cudaGetLastError();
  (void)cudaStreamDestroy(cs);
  if (kernels) *kernels = g_kernel_launches.load() - k0;
  if (!ok && exec) {
    (void)cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
  return exec;
}

std::string json_dump(const json::Value& v) { return json::dump(v); }

}  // namespace gfpdb
