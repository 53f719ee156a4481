// extern "C" boundary: status codes + thread-local error strings over the
// C++ operators and kernels. Nothing here computes on the CPU: every compute
// entry point ends in CUDA kernels, and a missing device is an error.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>

#include "../../include/gfpdb.h"
#include "host/handles.h"
#include "host/pop.h"
#include "kernels/launch.h"

using namespace gfpdb;

namespace {

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

std::vector<std::string> names_of(const char* const* names, int32_t n) {
  std::vector<std::string> out;
  for (int32_t i = 0; i < n; ++i) {
    if (names[i] == nullptr) fail(GFPDB_EINVAL, "null column name");
    out.emplace_back(names[i]);
  }
  return out;
}

void require(bool cond, const char* what) {
  if (!cond) fail(GFPDB_EINVAL, what);
}

}  // namespace

extern "C" {

const char* gfpdb_last_error(void) { return last_error().c_str(); }

int32_t gfpdb_version(void) { return 100; }

int32_t gfpdb_device_init(int32_t device) {
  return guarded([&] {
    GF_CUDA(cudaSetDevice(device));
    ensure_device();
  });
}

uint64_t gfpdb_kernel_launch_count(void) { return g_kernel_launches.load(); }

int32_t gfpdb_memcpy(void* dst, const void* src, int64_t n_bytes, int32_t kind, void* stream) {
  return guarded([&] {
    require(n_bytes >= 0, "negative copy size");
    cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice : kind == 2 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    require(kind >= 1 && kind <= 3, "copy kind must be 1, 2 or 3");
    if (stream == nullptr) {
      GF_CUDA(cudaMemcpy(dst, src, static_cast<size_t>(n_bytes), k));
    } else {
      GF_CUDA(cudaMemcpyAsync(dst, src, static_cast<size_t>(n_bytes), k, as_stream(stream)));
    }
    if (kind == 1) copy_counters().h2d += n_bytes;
    if (kind == 2) copy_counters().d2h += n_bytes;
  });
}

int32_t gfpdb_host_alloc(void** ptr, int64_t n_bytes) {
  return guarded([&] {
    require(ptr != nullptr && n_bytes >= 0, "bad host allocation request");
    GF_CUDA(cudaMallocHost(ptr, static_cast<size_t>(n_bytes > 0 ? n_bytes : 1)));
  });
}

int32_t gfpdb_host_free(void* ptr) {
  return guarded([&] { GF_CUDA(cudaFreeHost(ptr)); });
}

int32_t gfpdb_stream_synchronize(void* stream) {
  return guarded([&] { GF_CUDA(cudaStreamSynchronize(as_stream(stream))); });
}

int32_t gfpdb_profile_enable(int32_t enable) {
  return guarded([&] { prof_enable(enable != 0); });
}

int32_t gfpdb_profile_reset(void) {
  return guarded([&] { prof_reset(); });
}

int32_t gfpdb_profile_read(const char* kernel_name, int64_t* launches, double* total_ms, double* total_bytes) {
  return guarded([&] {
    require(kernel_name != nullptr && launches != nullptr && total_ms != nullptr && total_bytes != nullptr,
            "null argument");
    prof_read(kernel_name, launches, total_ms, total_bytes);
  });
}

int32_t gfpdb_profile_kernels(char* buf, int64_t buf_len) {
  return guarded([&] {
    require(buf != nullptr && buf_len > 0, "null buffer");
    std::string s = prof_kernels();
    if (static_cast<int64_t>(s.size()) + 1 > buf_len) fail(GFPDB_EINVAL, "buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
  });
}

// ------------------------------------------------------------------ filter

int32_t gfpdb_filter_compile(const char* predicate_json, const ArrowSchema* schema, gfpdb_filter** out) {
  return guarded([&] {
    require(predicate_json != nullptr && out != nullptr, "null argument");
    auto fields = import_schema(schema);
    auto f = std::make_unique<gfpdb_filter>();
    f->pred = compile_predicate(parse_expr_json(predicate_json), fields);
    *out = f.release();
  });
}

int32_t gfpdb_filter_evaluate(const gfpdb_filter* filter, const ArrowSchema* in_schema, const ArrowDeviceArray* in,
                              const char* const* project_columns, int32_t n_project, ArrowSchema* out_schema,
                              ArrowDeviceArray* out, void* stream) {
  return gfpdb_select(filter, 0, nullptr, nullptr, in_schema, in, project_columns, n_project, out_schema, out,
                      stream);
}

void gfpdb_filter_free(gfpdb_filter* filter) { delete filter; }

// ------------------------------------------------------------------- bloom

int32_t gfpdb_bloom_create(const ArrowSchema* schema, const ArrowDeviceArray* const* batches, int32_t n_batches,
                           const char* key_column, int32_t bits_per_key, int32_t num_hashes, gfpdb_bloom** out,
                           void* stream) {
  return guarded([&] {
    require(out != nullptr && key_column != nullptr && n_batches >= 0, "bad bloom_create arguments");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    std::vector<TupleSetPtr> keep;
    std::vector<const Column*> parts;
    for (int32_t i = 0; i < n_batches; ++i) {
      keep.push_back(import_tupleset(schema, batches[i], s));
      parts.push_back(keep.back()->column(key_column).get());
    }
    auto b = std::make_unique<gfpdb_bloom>();
    b->bloom = bloom_build(parts, bits_per_key, num_hashes, s);
    sync(s);  // borrowed inputs may be released after return
    *out = b.release();
  });
}

int32_t gfpdb_bloom_use(const gfpdb_bloom* bloom, const ArrowSchema* in_schema, const ArrowDeviceArray* in,
                        const char* key_column, ArrowSchema* out_schema, ArrowDeviceArray* out, void* stream) {
  const gfpdb_bloom* blooms[1] = {bloom};
  const char* cols[1] = {key_column};
  return gfpdb_select(nullptr, 1, blooms, cols, in_schema, in, nullptr, -1, out_schema, out, stream);
}

int32_t gfpdb_bloom_info(const gfpdb_bloom* bloom, int64_t* num_blocks, int64_t* num_keys, int32_t* valid,
                         int32_t* num_hashes, const void** device_blocks) {
  return guarded([&] {
    require(bloom != nullptr, "null bloom");
    if (num_blocks) *num_blocks = bloom->bloom->num_blocks;
    if (num_keys) *num_keys = bloom->bloom->num_keys;
    if (valid) *valid = bloom->bloom->valid ? 1 : 0;
    if (num_hashes) *num_hashes = bloom->bloom->num_hashes;
    if (device_blocks) *device_blocks = bloom->bloom->blocks->data();
  });
}

void gfpdb_bloom_free(gfpdb_bloom* bloom) { delete bloom; }

// ------------------------------------------------------------ fused select

int32_t gfpdb_select(const gfpdb_filter* filter, int32_t n_blooms, const gfpdb_bloom* const* blooms,
                     const char* const* bloom_key_columns, const ArrowSchema* in_schema, const ArrowDeviceArray* in,
                     const char* const* project_columns, int32_t n_project, ArrowSchema* out_schema,
                     ArrowDeviceArray* out, void* stream) {
  return guarded([&] {
    require(out_schema != nullptr && out != nullptr, "null output");
    require(n_blooms >= 0, "negative bloom count");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    auto ts = import_tupleset(in_schema, in, s);
    std::vector<BloomProbe> probes;
    for (int32_t i = 0; i < n_blooms; ++i) {
      require(blooms[i] != nullptr && bloom_key_columns[i] != nullptr, "null bloom or bloom key column");
      probes.push_back(BloomProbe{blooms[i]->bloom, bloom_key_columns[i]});
    }
    std::vector<std::string> proj;
    const bool all = n_project < 0 || project_columns == nullptr;
    if (!all) proj = names_of(project_columns, n_project);
    auto res = select_rows(*ts, filter ? &filter->pred : nullptr, probes, proj, all, s);
    export_tupleset(res, out_schema, out, false, s);
  });
}

// --------------------------------------------------------------- hash join

int32_t gfpdb_hashjoin_create(int32_t join_type, const char* build_key, const char* probe_key,
                              const char* const* needed_columns, int32_t n_needed, double load_factor,
                              gfpdb_hashjoin** out) {
  return guarded([&] {
    require(out != nullptr && build_key != nullptr && probe_key != nullptr, "null argument");
    if (join_type != GFPDB_JOIN_INNER) fail(GFPDB_EUNSUPPORTED, "only inner joins run on the GPU path");
    auto j = std::make_unique<gfpdb_hashjoin>();
    j->join_type = join_type;
    j->build_key = build_key;
    j->probe_key = probe_key;
    j->all_columns = needed_columns == nullptr || n_needed < 0;
    if (!j->all_columns) j->needed = names_of(needed_columns, n_needed);
    j->load_factor = load_factor > 0 ? load_factor : 0.5;
    *out = j.release();
  });
}

int32_t gfpdb_hashjoin_put_build(gfpdb_hashjoin* join, const ArrowSchema* schema, const ArrowDeviceArray* batch,
                                 void* stream) {
  return guarded([&] {
    require(join != nullptr, "null join");
    if (join->built) fail(GFPDB_EINVAL, "build input after finalize_build");
    ensure_device();
    // The batch outlives this call, so device inputs are copied.
    join->build.push_back(import_tupleset(schema, batch, as_stream(stream), true));
  });
}

int32_t gfpdb_hashjoin_finalize_build(gfpdb_hashjoin* join, void* stream) {
  return guarded([&] {
    require(join != nullptr, "null join");
    if (join->built) return;
    if (join->build.empty()) fail(GFPDB_EINVAL, "no build-side input");
    cudaStream_t s = as_stream(stream);
    join->table.build = TupleSet::concatenate(join->build, s);
    join->table.key_col = join->table.build->require_column(join->build_key);
    join_build_table(join->table, join->load_factor, s);
    join->build.clear();
    join->built = true;
  });
}

int32_t gfpdb_hashjoin_probe(gfpdb_hashjoin* join, const ArrowSchema* schema, const ArrowDeviceArray* batch,
                             ArrowSchema* out_schema, ArrowDeviceArray* out, void* stream) {
  return guarded([&] {
    require(join != nullptr && out != nullptr && out_schema != nullptr, "null argument");
    if (!join->built) fail(GFPDB_EINVAL, "probe before finalize_build");
    cudaStream_t s = as_stream(stream);
    auto ts = import_tupleset(schema, batch, s);
    const int pk = ts->require_column(join->probe_key);
    BufferPtr pidx, bidx;
    int64_t n = 0;
    join_probe_pairs(join->table, *ts, pk, &pidx, &bidx, &n, s);
    auto needed = [&](const std::string& c) {
      return join->all_columns || std::find(join->needed.begin(), join->needed.end(), c) != join->needed.end();
    };
    std::vector<GatherSpec> specs;
    std::vector<Field> fields;
    for (int i = 0; i < ts->num_columns(); ++i)
      if (needed(ts->field(i).name)) {
        fields.push_back(ts->field(i));
        specs.push_back(GatherSpec{ts->column(i).get(), pidx->as<int32_t>()});
      }
    const TupleSet& b = *join->table.build;
    for (int i = 0; i < b.num_columns(); ++i)
      if (needed(b.field(i).name)) {
        for (auto& f : fields)
          if (f.name == b.field(i).name) fail(GFPDB_EINVAL, "column '" + f.name + "' is on both join sides");
        fields.push_back(b.field(i));
        specs.push_back(GatherSpec{b.column(i).get(), bidx->as<int32_t>()});
      }
    auto cols = gather_columns(specs, n, s);
    export_tupleset(TupleSet::make(std::move(fields), std::move(cols), n), out_schema, out, false, s);
    sync(s);
  });
}

int32_t gfpdb_hashjoin_info(const gfpdb_hashjoin* join, int64_t* build_rows, int64_t* capacity, int64_t* max_probe) {
  return guarded([&] {
    require(join != nullptr, "null join");
    if (build_rows) *build_rows = join->built ? join->table.build->num_rows() : 0;
    if (capacity) *capacity = static_cast<int64_t>(join->table.capacity);
    if (max_probe) {
      *max_probe = 0;
      if (join->built) {
        DevStatus st;
        GF_CUDA(cudaMemcpy(&st, join->table.slots->as<char>() + join->table.capacity * 8, sizeof(st),
                           cudaMemcpyDeviceToHost));
        *max_probe = st.aux[0];
      }
    }
  });
}

void gfpdb_hashjoin_free(gfpdb_hashjoin* join) { delete join; }

// ---------------------------------------------------------------- group-by

int32_t gfpdb_group_create(const char* group_spec_json, gfpdb_group** out) {
  return guarded([&] {
    require(group_spec_json != nullptr && out != nullptr, "null argument");
    json::Value spec;
    try {
      spec = json::parse(group_spec_json);
    } catch (const std::exception& e) {
      fail(GFPDB_EINVAL, e.what());
    }
    std::vector<GroupAggregate> aggs;
    for (auto& a : spec.at("aggregates").array()) {
      GroupAggregate g;
      const std::string f = a.at("function").str();
      if (f == "SUM") g.fn = AGG_SUM;
      else if (f == "COUNT") g.fn = AGG_COUNT;
      else if (f == "MIN") g.fn = AGG_MIN;
      else if (f == "MAX") g.fn = AGG_MAX;
      else if (f == "AVG") g.fn = AGG_AVG;
      else fail(GFPDB_EUNSUPPORTED, "aggregate function '" + f + "'");
      g.name = a.at("name").str();
      if (a.contains("expr") && a.at("expr").kind != json::Value::Null) g.expr = parse_expr(a.at("expr"));
      else if (g.fn == AGG_COUNT) g.fn = AGG_COUNT_STAR;
      else fail(GFPDB_EINVAL, "aggregate '" + g.name + "' needs an expr");
      aggs.push_back(g);
    }
    auto g = std::make_unique<gfpdb_group>();
    g->table = group_table_create(spec.str_list("groupColumnNames"), aggs, spec.get_int("groupsHint", 0));
    *out = g.release();
  });
}

int32_t gfpdb_group_update(gfpdb_group* group, const ArrowSchema* schema, const ArrowDeviceArray* batch, void* stream) {
  return guarded([&] {
    require(group != nullptr, "null group");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    auto ts = import_tupleset(schema, batch, s);
    group_table_update(*group->table, *ts, s);
    sync(s);  // the batch is borrowed only for this call
  });
}

int32_t gfpdb_group_finalize(gfpdb_group* group, ArrowSchema* out_schema, ArrowDeviceArray* out, void* stream) {
  return guarded([&] {
    require(group != nullptr && out_schema != nullptr && out != nullptr, "null argument");
    cudaStream_t s = as_stream(stream);
    export_tupleset(group_table_finalize(*group->table, s), out_schema, out, false, s);
    sync(s);
  });
}

void gfpdb_group_free(gfpdb_group* group) { delete group; }

// --------------------------------------------------------------------- CSV

int32_t gfpdb_csv_read(const void* text, int64_t n_bytes, int32_t text_device_type, char delimiter, int32_t has_header,
                       const ArrowSchema* target_schema, const char* const* columns, int32_t n_columns,
                       ArrowSchema* out_schema, ArrowDeviceArray* out, void* stream) {
  return guarded([&] {
    require(text != nullptr || n_bytes == 0, "null text");
    require(out_schema != nullptr && out != nullptr, "null output");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    require(target_schema != nullptr && target_schema->format != nullptr &&
                std::strcmp(target_schema->format, "+s") == 0,
            "CSV target schema must be a struct");
    std::vector<CsvField> fields;
    for (int64_t i = 0; i < target_schema->n_children; ++i) {
      const ArrowSchema* c = target_schema->children[i];
      CsvField f;
      f.name = c->name ? c->name : "";
      const char* fmt = c->format;
      if (fmt != nullptr && std::strncmp(fmt, "d:", 2) == 0) {
        // decimal(precision,scale): parsed exactly into int64 scaled by 10^scale
        const char* comma = std::strchr(fmt, ',');
        require(comma != nullptr, "decimal format must be d:precision,scale");
        f.type = DType::Int64;
        f.decimal = true;
        f.scale = std::atoi(comma + 1);
        require(f.scale >= 0 && f.scale <= 9, "decimal scale must be in [0, 9]");
      } else {
        f.type = dtype_from_format(fmt);
      }
      fields.push_back(f);
    }
    std::vector<int> emit;
    if (columns == nullptr || n_columns < 0) {
      for (size_t i = 0; i < fields.size(); ++i) emit.push_back(static_cast<int>(i));
    } else {
      for (int32_t k = 0; k < n_columns; ++k) {
        int found = -1;
        for (size_t i = 0; i < fields.size(); ++i)
          if (fields[i].name == columns[k]) found = static_cast<int>(i);
        if (found < 0) fail(GFPDB_EINVAL, std::string("CSV column '") + columns[k] + "' is not in the schema");
        emit.push_back(found);
      }
    }
    const char* dtext = static_cast<const char*>(text);
    BufferPtr copy;
    if (text_device_type != ARROW_DEVICE_CUDA) {
      copy = make_buffer(n_bytes, s);
      memcpy_h2d(copy->data(), text, n_bytes, s);
      dtext = copy->as<char>();
    }
    auto res = csv_parse(dtext, n_bytes, delimiter, has_header != 0, fields, emit, s);
    export_tupleset(res, out_schema, out, false, s);
    sync(s);
  });
}

// ----------------------------------------------------------- plan execution

int32_t gfpdb_execute_plan(const char* plan_json, int32_t n_tables, const char* const* table_names,
                           const ArrowSchema* const* schemas, const ArrowDeviceArray* const* arrays,
                           int32_t result_to_host, ArrowSchema* out_schema, ArrowDeviceArray* out,
                           gfpdb_exec_stats* stats, void* stream) {
  return guarded([&] {
    require(plan_json != nullptr && out_schema != nullptr && out != nullptr, "null argument");
    const auto t0 = std::chrono::steady_clock::now();
    ensure_device();
    cudaStream_t s = as_stream(stream);
    const CopyCounters c0 = copy_counters();
    json::Value plan;
    try {
      plan = json::parse(plan_json);
    } catch (const std::exception& e) {
      fail(GFPDB_EINVAL, e.what());
    }
    std::map<std::string, pop::InputTable> inputs;
    for (int32_t i = 0; i < n_tables; ++i) {
      require(table_names[i] != nullptr, "null table name");
      pop::InputTable t;
      if (arrays[i]->device_type == ARROW_DEVICE_CUDA) {
        t.device = import_tupleset(schemas[i], arrays[i], s);
      } else {
        t.schema = schemas[i];
        t.array = arrays[i];
      }
      inputs[table_names[i]] = t;
    }
    auto ex = pop::build_execution(plan, s);
    ex->setInputs(std::move(inputs));
    auto result = ex->execute();
    export_tupleset(result, out_schema, out, result_to_host != 0, s);
    sync(s);
    if (stats != nullptr) {
      auto st = ex->stats();
      stats->kernel_launches = st.kernel_launches;
      stats->h2d_bytes = copy_counters().h2d - c0.h2d;
      stats->d2h_bytes = copy_counters().d2h - c0.d2h;
      stats->num_ops = st.num_ops;
      stats->messages = st.messages;
      stats->elapsed_ns =
          std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

int32_t gfpdb_plan_validate(const char* plan_json) {
  return guarded([&] {
    require(plan_json != nullptr, "null plan");
    json::Value plan;
    try {
      plan = json::parse(plan_json);
    } catch (const std::exception& e) {
      fail(GFPDB_EINVAL, e.what());
    }
    pop::validate_plan(plan);
  });
}

}  // extern "C"
