// C ABI of the request server (include/gfpdb.h, "request server").
#include <cstring>

#include "../../include/gfpdb.h"
#include "host/json.h"
#include "host/server.h"

using namespace gfpdb;

struct gfpdb_server {
  std::unique_ptr<serve::Server> impl;
};

namespace {

void require_ok(bool c, const char* msg) {
  if (!c) fail(GFPDB_EINVAL, msg);
}

serve::HostTable host_table(const ArrowSchema* schema, const ArrowDeviceArray* array) {
  require_ok(schema && array && schema->format && std::strcmp(schema->format, "+s") == 0,
             "a registered table is a struct array (ArrowSchema \"+s\")");
  require_ok(array->device_type == ARROW_DEVICE_CPU || array->device_type == ARROW_DEVICE_CUDA_HOST,
             "a registered table must live in host memory");
  const ArrowArray& top = array->array;
  require_ok(top.n_children == schema->n_children, "schema and array disagree on the number of columns");
  serve::HostTable t;
  t.rows = top.length;
  for (int64_t i = 0; i < schema->n_children; ++i) {
    const ArrowSchema* cs = schema->children[i];
    const ArrowArray* ca = top.children[i];
    require_ok(ca->length == top.length, "columns of a registered table must have the table's length");
    require_ok(ca->null_count == 0, "registered columns must not hold nulls");
    serve::HostColumn c;
    c.name = cs->name ? cs->name : "";
    c.type = dtype_from_format(cs->format);
    const int64_t off = ca->offset + top.offset;
    if (c.type == DType::Utf8) {
      c.offsets = static_cast<const int32_t*>(ca->buffers[1]) + off;
      c.values = ca->buffers[2];
    } else {
      c.values = static_cast<const char*>(ca->buffers[1]) + off * dtype_width(c.type);
    }
    t.cols.push_back(c);
  }
  return t;
}

}  // namespace

extern "C" {

int32_t gfpdb_server_create(const char* config_json, gfpdb_server** out) {
  return guarded([&] {
    require_ok(out != nullptr, "null output");
    serve::Config c;
    if (config_json != nullptr && config_json[0] != '\0') {
      json::Value v;
      try {
        v = json::parse(config_json);
      } catch (const std::exception& e) {
        fail(GFPDB_EINVAL, e.what());
      }
      c.device = static_cast<int>(v.get_int("device", c.device));
      c.workers = static_cast<int>(v.get_int("workers", c.workers));
      c.hbm_budget = static_cast<int64_t>(v.get_num("hbmBudgetBytes", static_cast<double>(c.hbm_budget)));
      c.cache_bytes = static_cast<int64_t>(v.get_num("cacheBytes", static_cast<double>(c.cache_bytes)));
      c.max_batch = static_cast<int>(v.get_int("maxBatch", c.max_batch));
      c.batching = v.get_bool("batching", c.batching);
      c.plan_streams = static_cast<int>(v.get_int("planStreams", c.plan_streams));
      c.graphs = v.get_bool("cudaGraphs", c.graphs);
      c.admission_timeout_ms = v.get_int("admissionTimeoutMs", c.admission_timeout_ms);
    }
    ensure_device();
    auto* s = new gfpdb_server();
    try {
      s->impl = std::make_unique<serve::Server>(c);
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
  });
}

int32_t gfpdb_server_register_table(gfpdb_server* server, const char* name, const ArrowSchema* schema,
                                    const ArrowDeviceArray* array) {
  return guarded([&] {
    require_ok(server != nullptr && name != nullptr, "null argument");
    server->impl->register_table(name, host_table(schema, array));
  });
}

int32_t gfpdb_server_submit(gfpdb_server* server, const char* request_json, uint64_t* ticket) {
  return guarded([&] {
    require_ok(server != nullptr && request_json != nullptr && ticket != nullptr, "null argument");
    *ticket = server->impl->submit(request_json);
  });
}

int32_t gfpdb_server_wait(gfpdb_server* server, uint64_t ticket, int64_t timeout_ms, ArrowSchema* out_schema,
                          ArrowDeviceArray* out, gfpdb_request_stats* stats) {
  int32_t rc = GFPDB_OK;
  const int32_t g = guarded([&] {
    require_ok(server != nullptr, "null server");
    rc = server->impl->wait(ticket, timeout_ms, out_schema, out, stats);
  });
  return g != GFPDB_OK ? g : rc;
}

int32_t gfpdb_server_get_stats(gfpdb_server* server, gfpdb_server_stats* out) {
  return guarded([&] {
    require_ok(server != nullptr && out != nullptr, "null argument");
    server->impl->stats(out);
  });
}

int32_t gfpdb_server_destroy(gfpdb_server* server) {
  return guarded([&] { delete server; });
}

}  // extern "C"
