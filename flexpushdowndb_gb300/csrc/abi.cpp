// extern "C" boundary: status codes + thread-local error strings over the
// C++ operators and kernels. Nothing here computes on the CPU: every compute
// entry point ends in CUDA kernels, and a missing device is an error.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "../../include/gfpdb.h"
#include "host/batchspec.h"
#include "host/handles.h"
#include "host/parquet_meta.h"
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

// ---- captured plans
//
// A plan run with "cudaGraph": true is captured once per (device, plan text,
// input buffers) into a CUDA graph whose allocations come from a bump arena
// sized from an ordinary run, so every replay finds its inputs, outputs and
// status blocks at the same addresses. A replay is one graph launch plus the
// same end-of-plan status checks as an ordinary deferred run.
struct CapturedPlan {
  std::unique_ptr<Arena> arena;
  cudaGraphExec_t exec = nullptr;
  // The graph ends with one kernel that packs every status block and the
  // result (row count and columns) straight into this page-locked buffer,
  // which the device reaches through unified addressing.
  char* pinned = nullptr;
  int64_t pinned_bytes = 0;
  std::vector<int64_t> status_off;
  int64_t count_off = -1;  // result row count (deferred result), else exact_rows
  int64_t exact_rows = 0;
  std::vector<std::vector<int64_t>> col_off;  // per result column, its buffers
  TupleSetPtr result;
  std::vector<DeferredCheck> checks;
  uint64_t kernels = 0;
  bool in_flight = false;  // launched and not yet finished
  int64_t num_ops = 0, messages = 0, h2d = 0;
  bool capturable = true;
  cudaEvent_t ev[2] = {nullptr, nullptr};  // around a replay: its device time
  ~CapturedPlan() {
    for (auto e : ev)
      if (e) (void)cudaEventDestroy(e);
    if (exec) (void)cudaGraphExecDestroy(exec);
    if (pinned) (void)cudaFreeHost(pinned);
  }
};

// The end of a captured plan, issued on the capturing stream: one pack of
// every status block and of the result into the page-locked buffer.
void capture_epilogue(CapturedPlan& cp, cudaStream_t cs) {
  std::vector<CopySpan> spans;
  int64_t off = 0;
  auto add = [&](const void* src, int64_t bytes) {
    const int64_t o = off;
    spans.push_back(CopySpan{src, bytes, o});
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  for (auto& c : cp.checks) cp.status_off.push_back(add(c.status, sizeof(DevStatus)));
  const TupleSet& r = *cp.result;
  const int64_t cap = r.num_rows();
  if (r.exact()) cp.exact_rows = cap;
  else cp.count_off = add(r.rows_dev(), sizeof(int64_t));
  for (int i = 0; i < r.num_columns(); ++i) {
    const auto& c = r.column(i);
    if (c->type == DType::Utf8) {
      if (!c->data_buf) fail(GFPDB_EUNSUPPORTED, "captured plan result without its own string buffer");
      const int64_t o1 = add(c->offsets, (cap + 1) * 4);
      const int64_t o2 = add(c->data, c->data_buf->size());
      cp.col_off.push_back({o1, o2});
    } else {
      cp.col_off.push_back({add(c->data, cap * dtype_width(c->type))});
    }
  }
  cp.pinned_bytes = off > 0 ? off : 256;
  // page-locked allocation is not a stream operation: allowed mid-capture
  // under the relaxed mode
  cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
  GF_CUDA(cudaThreadExchangeStreamCaptureMode(&mode));
  const cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&cp.pinned), cp.pinned_bytes);
  GF_CUDA(cudaThreadExchangeStreamCaptureMode(&mode));
  GF_CUDA(e);
  pack_spans(spans, cp.pinned, cs);
}

std::mutex g_graph_mu;
std::map<std::string, std::shared_ptr<CapturedPlan>> g_graphs;

std::string plan_key(const char* plan_json, int32_t n_tables, const char* const* names,
                     const ArrowDeviceArray* const* arrays) {
  std::string key = std::to_string(current_device()) + "|" + plan_json;
  for (int32_t i = 0; i < n_tables; ++i) {
    const ArrowArray& a = arrays[i]->array;
    key += "|" + std::string(names[i]) + ":" + std::to_string(arrays[i]->device_type) + ":" +
           std::to_string(a.length) + ":" + std::to_string(a.offset);
    for (int64_t c = 0; c < a.n_children; ++c)
      for (int64_t b = 0; b < a.children[c]->n_buffers; ++b)
        key += ":" + std::to_string(reinterpret_cast<uintptr_t>(a.children[c]->buffers[b]));
  }
  return key;
}

struct ArenaGuard {
  explicit ArenaGuard(Arena* a) { set_thread_arena(a); }
  ~ArenaGuard() { set_thread_arena(nullptr); }
};

std::shared_ptr<CapturedPlan> capture_plan(const json::Value& plan, const std::map<std::string, pop::InputTable>& inputs,
                                           int64_t arena_bytes, const int64_t fill_bytes[2][2]) {
  auto cp = std::make_shared<CapturedPlan>();
  cudaStream_t cs = nullptr;
  GF_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { (void)cudaStreamDestroy(s); }
  } sg{cs};
  // The arena outlives the capture stream: allocate it on the legacy stream.
  cp->arena = std::make_unique<Arena>(arena_bytes, nullptr);
  sync(nullptr);
  const uint64_t k0 = g_kernel_launches.load();
  // host bytes a replay moves: the captured copies, and the page-locked
  // columns its kernels read in place (their full size: an upper bound)
  const int64_t h2d0 = copy_counters().h2d + copy_counters().in_place;
  cudaGraph_t graph = nullptr;
  bool ok = true;
  // The buffers the operators want pre-filled (sized by the ordinary run,
  // with room to spare) come from regions that the graph fills first: the
  // small ones on the capturing stream, the large ones on a side stream.
  FillPool pool;
  for (int t = 0; t < 2; ++t)
    for (int k = 0; k < 2; ++k) {
      if (fill_bytes[t][k] <= 0) continue;
      pool.size[t][k] = fill_bytes[t][k] + fill_bytes[t][k] / 4 + 4096;
      pool.base[t][k] = static_cast<char*>(cp->arena->take(pool.size[t][k]));
    }
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr;
  GF_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  GF_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  GF_CUDA(cudaEventCreateWithFlags(&pool.large_ready, cudaEventDisableTiming));
  struct SideGuard {
    cudaStream_t s;
    cudaEvent_t a, b;
    ~SideGuard() {
      (void)cudaEventDestroy(a);
      (void)cudaEventDestroy(b);
      (void)cudaStreamDestroy(s);
    }
  } side_guard{side, fork, pool.large_ready};
  {
    ArenaGuard ag(cp->arena.get());
    struct PoolGuard {
      explicit PoolGuard(FillPool* p) { set_thread_fill_pool(p); }
      ~PoolGuard() { set_thread_fill_pool(nullptr); }
    } pg(&pool);
    GF_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
      // one fill kernel per size class (kernel nodes follow each other more
      // closely than memset nodes)
      const FillSpan small[2] = {{pool.base[0][0], pool.size[0][0], 0, 0}, {pool.base[0][1], pool.size[0][1], 0xFF, 0}};
      const FillSpan large[2] = {{pool.base[1][0], pool.size[1][0], 0, 0}, {pool.base[1][1], pool.size[1][1], 0xFF, 0}};
      fill_regions(small, 2, cs);
      GF_CUDA(cudaEventRecord(fork, cs));
      GF_CUDA(cudaStreamWaitEvent(side, fork, 0));
      fill_regions(large, 2, side);
      GF_CUDA(cudaEventRecord(pool.large_ready, side));
      auto ex = pop::build_execution(plan, cs);
      ex->setInputs(inputs);
      ex->setDeferred(true);
      ex->setCapturing(true);
      cp->result = ex->execute();
      cp->checks = ex->takeCapturedChecks();
      cp->num_ops = ex->stats().num_ops;
      cp->messages = ex->stats().messages;
      capture_epilogue(*cp, cs);
      GF_CUDA(cudaStreamWaitEvent(cs, pool.large_ready, 0));  // the side stream rejoins
    } catch (const std::exception&) {
      ok = false;  // something in the plan needs the host mid-run
    }
    const cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (e != cudaSuccess) ok = false;
  }
  (void)cudaGetLastError();
  if (ok && graph != nullptr && cudaGraphInstantiate(&cp->exec, graph, 0) != cudaSuccess) ok = false;
  if (graph != nullptr) (void)cudaGraphDestroy(graph);
  (void)cudaGetLastError();
  cp->h2d = copy_counters().h2d + copy_counters().in_place - h2d0;
  cp->kernels = g_kernel_launches.load() - k0;
  if (!ok) {
    cp->capturable = false;
    cp->result.reset();
    cp->checks.clear();
  }
  return cp;
}

// ---- batched star queries: prepared batches (and their graphs), cached.

struct BatchEntry {
  StarBatch batch;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;
  std::vector<CopySpan> spans;  // a prepared batch's result pack
  ~BatchEntry() {
    if (exec) (void)cudaGraphExecDestroy(exec);
  }
};

std::mutex g_batch_mu;
std::map<std::string, std::shared_ptr<BatchEntry>> g_batches;

std::shared_ptr<BatchEntry> find_batch(const std::string& key) {
  std::lock_guard<std::mutex> lk(g_batch_mu);
  auto it = g_batches.find(key);
  return it == g_batches.end() ? nullptr : it->second;
}

void remember_batch(const std::string& key, std::shared_ptr<BatchEntry> be) {
  std::lock_guard<std::mutex> lk(g_batch_mu);
  if (g_batches.size() >= 64) g_batches.clear();  // bounded cache
  g_batches[key] = std::move(be);
}

void clear_batches() {
  std::lock_guard<std::mutex> lk(g_batch_mu);
  g_batches.clear();
}

// The input tables of a batched star query: device tables are used in
// place; host tables get device copies here, and every run refreshes the
// columns the batch reads from the host buffers (host_cols).
struct BatchInputs {
  std::map<std::string, TupleSetPtr> tables;
  std::vector<StarBatchHostColumn> host_cols;
  bool pageable = false;  // some host table is in pageable memory
};

BatchInputs import_batch_inputs(int32_t n_tables, const char* const* table_names, const ArrowSchema* const* schemas,
                                const ArrowDeviceArray* const* arrays, cudaStream_t s) {
  BatchInputs in;
  for (int32_t i = 0; i < n_tables; ++i) {
    require(table_names[i] != nullptr && arrays[i] != nullptr, "null table");
    const int32_t dt = arrays[i]->device_type;
    if (dt != ARROW_DEVICE_CUDA && dt != ARROW_DEVICE_CPU && dt != ARROW_DEVICE_CUDA_HOST)
      fail(GFPDB_EUNSUPPORTED, "unsupported ArrowDeviceArray device_type " + std::to_string(dt));
    TupleSetPtr t = import_tupleset(schemas[i], arrays[i], s, false);
    if (dt != ARROW_DEVICE_CUDA) {
      in.pageable |= dt == ARROW_DEVICE_CPU;
      const ArrowArray& a = arrays[i]->array;
      for (int c = 0; c < t->num_columns(); ++c) {
        const auto& col = t->column(c);
        if (col->type == DType::Utf8) continue;
        const int w = dtype_width(col->type);
        const ArrowArray* ch = a.children[c];
        const char* src = static_cast<const char*>(ch->buffers[1]) + (ch->offset + a.offset) * w;
        if (col->data != src) in.host_cols.push_back(StarBatchHostColumn{col->data, src, t->num_rows() * w});
      }
    }
    in.tables[table_names[i]] = t;
  }
  sync(s);  // the first copies have landed
  return in;
}

std::shared_ptr<BatchEntry> make_batch(const json::Value& spec, const std::map<std::string, TupleSetPtr>& tables,
                                       bool use_graph, cudaStream_t s,
                                       std::vector<StarBatchHostColumn> host_cols = {}) {
  auto be = std::make_shared<BatchEntry>();
  be->batch.set_host_columns(std::move(host_cols));
  StarBatchSpec& sp = be->batch.spec();
  auto table = [&](const std::string& name) {
    auto it = tables.find(name);
    if (it == tables.end()) fail(GFPDB_EINVAL, "batched star query names table '" + name + "' which was not passed");
    return it->second;
  };
  parse_star_batch_spec(spec, sp);
  if (sp.queries.empty()) fail(GFPDB_EINVAL, "a batched star query needs \"queries\"");
  for (auto& n : sp.fact_tables) be->batch.parts().push_back(table(n));
  for (auto& d : sp.dims) be->batch.dim_tables().push_back(table(d.table));
  be->batch.prepare(s);
  if (use_graph) be->exec = capture_star_batch(be->batch, &be->kernels);
  return be;
}

// A device copy of the first n rows of an arena-backed result (the next
// replay reuses the arena).
TupleSetPtr device_copy(const TupleSet& r, int64_t n, cudaStream_t s) {
  std::vector<ColumnPtr> cols;
  for (int i = 0; i < r.num_columns(); ++i) {
    const auto& c = r.column(i);
    if (c->type == DType::Utf8) {
      Column part = *c;
      part.length = n;
      cols.push_back(concat_utf8({&part}, s));
    } else {
      const int w = dtype_width(c->type);
      auto b = make_buffer(n * w, s);
      if (n > 0) GF_CUDA(cudaMemcpyAsync(b->data(), c->data, n * w, cudaMemcpyDeviceToDevice, s));
      cols.push_back(make_fixed_column(c->type, n, b));
    }
  }
  return TupleSet::make(r.fields(), std::move(cols), n);
}

// Replay a captured plan. Returns false when a deferred output overflowed
// (the caller then runs the plan with exact sizes).
// One replay: launch, wait, check every status. Returns false when a
// deferred output overflowed; else *n_rows is the result's row count (its
// values in cp.pinned).
// A replay in two halves: the launch (the graph between two events on the
// stream) and the finish (wait for the second event, read the statuses the
// graph packed into page-locked memory). Between them the caller may launch
// other work, another prepared plan's replay included.
void replay_launch(CapturedPlan& cp, cudaStream_t s) {
  // one replay of a captured plan at a time: a second would share its
  // scratch, result buffers and events
  if (cp.in_flight)
    fail(GFPDB_EINVAL, "this captured plan is already running; prepare the second copy with another \"graphInstance\"");
  if (cp.ev[0] == nullptr) {
    GF_CUDA(cudaEventCreate(&cp.ev[0]));
    GF_CUDA(cudaEventCreate(&cp.ev[1]));
  }
  GF_CUDA(cudaEventRecord(cp.ev[0], s));
  GF_CUDA(cudaGraphLaunch(cp.exec, s));
  GF_CUDA(cudaEventRecord(cp.ev[1], s));
  cp.in_flight = true;
  count_launch(cp.kernels);
}

// False when a deferred size overflowed: the caller re-runs the plan with
// exact sizes.
bool replay_finish(CapturedPlan& cp, cudaStream_t s, int64_t* device_ns, int64_t* n_rows) {
  // The replay is over for the plan's bookkeeping on every exit, a failed
  // completion query included: a later launch must not be refused as
  // "already running".
  struct InFlightReset {
    CapturedPlan& cp;
    ~InFlightReset() { cp.in_flight = false; }
  } in_flight_reset{cp};
  // A replay is short: poll its end instead of sleeping in a blocking wait,
  // which would add the thread's wake-up to every query; after about two
  // milliseconds fall back to the blocking wait.
  {
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
      const cudaError_t q = cudaEventQuery(cp.ev[1]);
      if (q == cudaSuccess) break;
      if (q != cudaErrorNotReady) GF_CUDA(q);
      if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(2000)) {
        sync(s);
        break;
      }
    }
  }
  float ms = 0;
  GF_CUDA(cudaEventElapsedTime(&ms, cp.ev[0], cp.ev[1]));
  *device_ns = static_cast<int64_t>(static_cast<double>(ms) * 1e6);
  copy_counters().h2d += cp.h2d;
  copy_counters().d2h += cp.pinned_bytes;
  bool fits = true;
  for (size_t i = 0; i < cp.checks.size(); ++i) {
    const DevStatus* st = reinterpret_cast<const DevStatus*>(cp.pinned + cp.status_off[i]);
    raise_device_status(*st, cp.checks[i].where);
    if (cp.checks[i].capacity > 0 && st->value > cp.checks[i].capacity) fits = false;
  }
  if (!fits) return false;
  const TupleSet& r = *cp.result;
  const int64_t n = cp.count_off >= 0 ? *reinterpret_cast<const int64_t*>(cp.pinned + cp.count_off) : cp.exact_rows;
  if (n < 0 || n > r.num_rows()) fail(GFPDB_EDEVICE, "captured plan produced an out-of-range row count");
  *n_rows = n;
  return true;
}

bool replay_graph(CapturedPlan& cp, cudaStream_t s, int64_t* device_ns, int64_t* n_rows) {
  replay_launch(cp, s);
  return replay_finish(cp, s, device_ns, n_rows);
}

bool replay_plan(CapturedPlan& cp, bool to_host, ArrowSchema* out_schema, ArrowDeviceArray* out, cudaStream_t s,
                 int64_t* device_ns) {
  int64_t n = 0;
  if (!replay_graph(cp, s, device_ns, &n)) return false;
  const TupleSet& r = *cp.result;
  if (to_host) {
    std::vector<std::vector<const void*>> bufs;
    for (auto& offs : cp.col_off) {
      std::vector<const void*> b;
      for (int64_t o : offs) b.push_back(cp.pinned + o);
      bufs.push_back(b);
    }
    export_host_columns(r.fields(), n, bufs, out_schema, out);
  } else {
    export_tupleset(device_copy(r, n, s), out_schema, out, false, s);
    sync(s);
  }
  return true;
}

}  // namespace

// A plan bound to its inputs (gfpdb_plan_prepare).
struct gfpdb_prepared {
  std::string plan;
  std::vector<std::string> names;
  std::vector<const char*> name_ptrs;
  std::vector<const ArrowSchema*> schemas;
  std::vector<const ArrowDeviceArray*> arrays;
  bool graph = false;
  std::string key;                                // the captured-plan cache key
  std::shared_ptr<CapturedPlan> cp;               // once captured
  ArrowSchema res_s{};                            // the last non-replay run's exported result
  ArrowDeviceArray res_a{};
  bool has_res = false;
  bool last_replay = false;
  int64_t generation = 0;
  // a launched run not yet waited for: none, a graph replay in flight, or a
  // run that completed inside the launch (the first runs, an uncaptured plan)
  enum Pending { kNone, kReplay, kDone } pending = kNone;
  void* stream = nullptr;
  std::chrono::steady_clock::time_point t0;
  gfpdb_exec_stats done_stats{};
  int64_t rows = 0;

  void find_capture() {
    if (!graph || cp) return;
    std::lock_guard<std::mutex> lk(g_graph_mu);
    auto it = g_graphs.find(key);
    if (it != g_graphs.end()) cp = it->second;
  }

  void release_result() {
    if (!has_res) return;
    if (res_a.array.release) res_a.array.release(&res_a.array);
    if (res_s.release) res_s.release(&res_s);
    has_res = false;
  }
  ~gfpdb_prepared() { release_result(); }
};

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

int64_t gfpdb_thread_device_alloc_bytes(void) { return thread_alloc_bytes(); }

int32_t gfpdb_result_layout(const ArrowSchema* schema, const ArrowDeviceArray* array, int32_t max_columns,
                            int64_t* n_rows, int32_t* n_columns, int32_t* device_type, char* names,
                            int64_t names_capacity, const void** values, const void** offsets) {
  return guarded([&] {
    require(schema != nullptr && array != nullptr && n_rows != nullptr && n_columns != nullptr &&
                device_type != nullptr && names != nullptr && values != nullptr && offsets != nullptr,
            "null argument");
    const ArrowArray& a = array->array;
    require(schema->n_children == a.n_children, "schema and array disagree on the column count");
    require(a.n_children <= max_columns, "more columns than max_columns");
    *n_rows = a.length;
    *n_columns = static_cast<int32_t>(a.n_children);
    *device_type = array->device_type;
    int64_t at = 0;
    auto put = [&](const char* s) {
      const int64_t len = static_cast<int64_t>(std::strlen(s)) + 1;
      require(at + len <= names_capacity, "column names exceed names_capacity");
      std::memcpy(names + at, s, static_cast<size_t>(len));
      at += len;
    };
    for (int64_t i = 0; i < a.n_children; ++i) {
      const ArrowSchema* cs = schema->children[i];
      const ArrowArray* ca = a.children[i];
      put(cs->name != nullptr ? cs->name : "");
      put(cs->format);
      const bool utf8 = std::strcmp(cs->format, "u") == 0;
      if (ca->null_count != 0 && ca->buffers[0] != nullptr)
        fail(GFPDB_EUNSUPPORTED, std::string("column '") + (cs->name ? cs->name : "") +
                                     "' holds nulls; the layout carries values only");
      values[i] = ca->buffers[utf8 ? 2 : 1];
      offsets[i] = utf8 ? ca->buffers[1] : nullptr;
    }
  });
}

void gfpdb_result_release(ArrowSchema* schema, ArrowDeviceArray* array) {
  if (array != nullptr && array->array.release != nullptr) array->array.release(&array->array);
  if (schema != nullptr && schema->release != nullptr) schema->release(schema);
}

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
                           const char* const* key_columns, int32_t n_keys, int32_t bits_per_key, int32_t num_hashes,
                           gfpdb_bloom** out, void* stream) {
  return guarded([&] {
    require(out != nullptr && key_columns != nullptr && n_batches >= 0, "bad bloom_create arguments");
    if (n_keys < 1 || n_keys > kMaxKeyColumns) fail(GFPDB_EINVAL, "a bloom filter key has 1 to 8 columns");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    const std::vector<std::string> keys = names_of(key_columns, n_keys);
    std::vector<TupleSetPtr> keep;
    std::vector<const Column*> parts;
    for (int32_t i = 0; i < n_batches; ++i) {
      TupleSetPtr t = import_tupleset(schema, batches[i], s);
      // several key columns: the filter holds their composite
      if (n_keys > 1) t = with_composite_key(t, keys, kBuildKeyColumn, "", s);
      keep.push_back(t);
      parts.push_back(t->column(n_keys > 1 ? std::string(kBuildKeyColumn) : keys[0]).get());
    }
    auto b = std::make_unique<gfpdb_bloom>();
    b->key_columns = n_keys;
    b->bloom = bloom_build(parts, bits_per_key, num_hashes, s);
    sync(s);  // borrowed inputs may be released after return
    *out = b.release();
  });
}

int32_t gfpdb_bloom_use(const gfpdb_bloom* bloom, const ArrowSchema* in_schema, const ArrowDeviceArray* in,
                        const char* const* key_columns, int32_t n_keys, ArrowSchema* out_schema,
                        ArrowDeviceArray* out, void* stream) {
  if (bloom != nullptr && key_columns != nullptr && n_keys == 1 && bloom->key_columns == 1) {
    const gfpdb_bloom* blooms[1] = {bloom};
    return gfpdb_select(nullptr, 1, blooms, key_columns, in_schema, in, nullptr, -1, out_schema, out, stream);
  }
  return guarded([&] {
    require(bloom != nullptr && key_columns != nullptr && out_schema != nullptr && out != nullptr, "null argument");
    if (n_keys != bloom->key_columns)
      fail(GFPDB_EINVAL, "the filter was built over " + std::to_string(bloom->key_columns) + " key columns, not " +
                             std::to_string(n_keys));
    ensure_device();
    cudaStream_t s = as_stream(stream);
    TupleSetPtr ts = import_tupleset(in_schema, in, s);
    std::vector<std::string> all;
    for (int i = 0; i < ts->num_columns(); ++i) all.push_back(ts->field(i).name);
    TupleSetPtr keyed = with_composite_key(ts, names_of(key_columns, n_keys), kProbeKeyColumn, "", s);
    TupleSetPtr r = select_rows(*keyed, nullptr, {BloomProbe{bloom->bloom, kProbeKeyColumn}}, all, false, s);
    export_tupleset(resolved(r, s), out_schema, out, false, s);
    sync(s);
  });
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

// ----------------------------------------------------------------- shuffle

int32_t gfpdb_shuffle(const ArrowSchema* in_schema, const ArrowDeviceArray* in, const char* const* key_columns,
                      int32_t n_keys, int64_t num_slots, ArrowSchema* out_schema, ArrowDeviceArray* out,
                      int64_t* slot_offsets, void* stream) {
  return guarded([&] {
    require(key_columns != nullptr && out_schema != nullptr && out != nullptr && slot_offsets != nullptr,
            "null argument");
    require(n_keys >= 1 && n_keys <= kMaxKeyColumns, "a shuffle key has 1 to 8 columns");
    require(num_slots >= 1 && num_slots <= kShuffleMaxSlots, "shuffle slots must be 1 to 1024");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    TupleSetPtr ts = import_tupleset(in_schema, in, s);
    ShuffleResult r = shuffle_rows(ts, names_of(key_columns, n_keys), num_slots, s);
    export_tupleset(r.rows, out_schema, out, false, s);
    std::copy(r.offsets.begin(), r.offsets.end(), slot_offsets);
  });
}

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

int32_t gfpdb_hashjoin_create(int32_t join_type, const char* const* build_keys, const char* const* probe_keys,
                              int32_t n_keys, const char* const* needed_columns, int32_t n_needed,
                              double load_factor, gfpdb_hashjoin** out) {
  return guarded([&] {
    require(out != nullptr && build_keys != nullptr && probe_keys != nullptr, "null argument");
    if (n_keys < 1 || n_keys > kMaxKeyColumns) fail(GFPDB_EINVAL, "a join key has 1 to 8 columns");
    if (join_type < GFPDB_JOIN_INNER || join_type > GFPDB_JOIN_RIGHT_SEMI)
      fail(GFPDB_EINVAL, "join type " + std::to_string(join_type));
    if (join_type != GFPDB_JOIN_INNER && n_keys != 1)
      fail(GFPDB_EUNSUPPORTED, "outer and semi joins take one key column per side");
    auto j = std::make_unique<gfpdb_hashjoin>();
    j->join_type = join_type;
    j->build_keys = names_of(build_keys, n_keys);
    j->probe_keys = names_of(probe_keys, n_keys);
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
    join->table = pop::build_join_table(TupleSet::concatenate(join->build, s), join->build_keys, join->load_factor, s,
                                        pop::join_kind_marks(static_cast<pop::JoinKind>(join->join_type)));
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
    if (join->probe_fields.empty()) join->probe_fields = ts->fields();
    // output: the probe side's needed columns, then the build side's
    // (HashJoinArrowKernel.cpp:148-162); every column when none are named
    std::vector<std::string> proj;
    if (join->all_columns) {
      for (int i = 0; i < ts->num_columns(); ++i) proj.push_back(ts->field(i).name);
      const TupleSet& b = *join->table.build;
      for (int i = 0; i < b.num_columns(); ++i)
        if (!is_internal_key_column(b.field(i).name)) proj.push_back(b.field(i).name);
    } else {
      proj = join->needed;
    }
    const auto kind = static_cast<pop::JoinKind>(join->join_type);
    TupleSetPtr r = pop::join_probe_kind("hash join", kind, join->table, proj, join->probe_keys, ts, s);
    if (!r) {  // LEFT_SEMI: rows come from gfpdb_hashjoin_finish
      std::vector<Field> none;
      r = TupleSet::make_empty(none, s);
    }
    export_tupleset(resolved(r, s), out_schema, out, false, s);
    sync(s);
  });
}

int32_t gfpdb_hashjoin_finish(gfpdb_hashjoin* join, const ArrowSchema* probe_schema, ArrowSchema* out_schema,
                              ArrowDeviceArray* out, void* stream) {
  return guarded([&] {
    require(join != nullptr && out != nullptr && out_schema != nullptr, "null argument");
    if (!join->built) fail(GFPDB_EINVAL, "finish before finalize_build");
    cudaStream_t s = as_stream(stream);
    std::vector<Field> pf = join->probe_fields;
    if (pf.empty() && probe_schema != nullptr) pf = import_schema(probe_schema);
    std::vector<std::string> proj;
    if (!join->all_columns) proj = join->needed;
    const auto kind = static_cast<pop::JoinKind>(join->join_type);
    TupleSetPtr r = pop::join_finish_kind("hash join", kind, join->table, pf, proj, s);
    if (!r) {
      std::vector<Field> none;
      r = TupleSet::make_empty(none, s);
    }
    export_tupleset(r, out_schema, out, false, s);
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
        GF_CUDA(cudaMemcpy(&st, join->table.status->data(), sizeof(st), cudaMemcpyDeviceToHost));
        *max_probe = st.aux[0];
      }
    }
  });
}

int32_t gfpdb_hashjoin_clear(gfpdb_hashjoin* join) {
  return guarded([&] {
    require(join != nullptr, "null argument");
    join->build.clear();
    join->table = JoinTable{};
    join->probe_fields.clear();
    join->built = false;
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
    std::vector<GroupAggregate> aggs = pop::parse_aggregates(spec.at("aggregates"));
    auto g = std::make_unique<gfpdb_group>();
    g->group_cols = spec.str_list("groupColumnNames");
    g->aggs = aggs;
    g->hint = spec.get_int("groupsHint", 0);
    g->table = group_table_create(g->group_cols, g->aggs, g->hint);
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

int32_t gfpdb_group_clear(gfpdb_group* group) {
  return guarded([&] {
    require(group != nullptr, "null argument");
    group->table = group_table_create(group->group_cols, group->aggs, group->hint);
  });
}

void gfpdb_group_free(gfpdb_group* group) { delete group; }

// ----------------------------------------------------------------- Parquet

int32_t gfpdb_parquet_read(const void* file, int64_t n_bytes, const char* const* columns, int32_t n_columns,
                           int64_t start_pos, int64_t end_pos, ArrowSchema* out_schema, ArrowDeviceArray* out,
                           void* stream) {
  return guarded([&] {
    require(file != nullptr && out_schema != nullptr && out != nullptr, "null argument");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    std::vector<std::string> names;
    if (columns != nullptr && n_columns >= 0) names = names_of(columns, n_columns);
    auto ts = parquet_read(static_cast<const uint8_t*>(file), n_bytes, names, start_pos, end_pos, s);
    export_tupleset(ts, out_schema, out, false, s);
  });
}

int32_t gfpdb_parquet_layout(const void* file, int64_t n_bytes, const char* const* columns, int32_t n_columns,
                             int64_t start_pos, int64_t end_pos, char* out_json, int64_t capacity, int64_t* needed) {
  return guarded([&] {
    require(file != nullptr && needed != nullptr && n_bytes >= 0, "null argument");
    std::vector<std::string> names;
    if (columns != nullptr && n_columns >= 0) names = names_of(columns, n_columns);
    const parquet::Layout L =
        parquet::read_layout(static_cast<const uint8_t*>(file), n_bytes, names, start_pos, end_pos);
    auto num = [](int64_t v) {
      json::Value x;
      x.kind = json::Value::Number;
      x.is_integer = true;
      x.i = v;
      return x;
    };
    auto str = [](const std::string& v) {
      json::Value x;
      x.kind = json::Value::String;
      x.s = v;
      return x;
    };
    auto obj = [] {
      json::Value x;
      x.kind = json::Value::Object;
      return x;
    };
    auto arr = [] {
      json::Value x;
      x.kind = json::Value::Array;
      return x;
    };
    json::Value out = obj(), cols = arr(), groups = arr(), chunks = arr(), pages = arr();
    for (const auto& c : L.columns) {
      json::Value o = obj();
      o.o.emplace_back("name", str(c.name));
      o.o.emplace_back("type", str(dtype_name(c.dtype)));
      o.o.emplace_back("physicalType", num(c.physical));
      json::Value req;
      req.kind = json::Value::Bool;
      req.b = c.repetition == 0;
      o.o.emplace_back("required", req);
      cols.a.push_back(o);
    }
    for (const auto& g : L.row_groups) {
      json::Value o = obj();
      o.o.emplace_back("offset", num(g.offset));
      o.o.emplace_back("rows", num(g.rows));
      groups.a.push_back(o);
    }
    for (const auto& c : L.chunks) {
      json::Value o = obj();
      o.o.emplace_back("begin", num(c.begin));
      o.o.emplace_back("end", num(c.end));
      chunks.a.push_back(o);
    }
    for (const auto& p : L.pages) {
      json::Value o = obj();
      o.o.emplace_back("column", num(p.column));
      o.o.emplace_back("chunk", num(p.chunk));
      o.o.emplace_back("pageType", num(p.type));
      o.o.emplace_back("encoding", num(p.encoding));
      o.o.emplace_back("codec", num(p.codec));
      o.o.emplace_back("offset", num(p.data_offset));
      o.o.emplace_back("compressedBytes", num(p.compressed));
      o.o.emplace_back("uncompressedBytes", num(p.uncompressed));
      o.o.emplace_back("numValues", num(p.num_values));
      o.o.emplace_back("firstRow", num(p.first_row));
      pages.a.push_back(o);
    }
    out.o.emplace_back("numRows", num(L.num_rows));
    out.o.emplace_back("columns", cols);
    out.o.emplace_back("rowGroups", groups);
    out.o.emplace_back("chunks", chunks);
    out.o.emplace_back("pages", pages);
    const std::string text = json::dump(out);
    *needed = static_cast<int64_t>(text.size()) + 1;
    if (out_json == nullptr || capacity < *needed) fail(GFPDB_EINVAL, "output buffer too small (see *needed)");
    std::memcpy(out_json, text.c_str(), text.size() + 1);
  });
}

int32_t gfpdb_parquet_read_file(const char* path, const char* const* columns, int32_t n_columns, int64_t start_pos,
                                int64_t end_pos, ArrowSchema* out_schema, ArrowDeviceArray* out, void* stream) {
  return guarded([&] {
    require(path != nullptr && out_schema != nullptr && out != nullptr, "null argument");
    ensure_device();
    cudaStream_t s = as_stream(stream);
    std::vector<std::string> names;
    if (columns != nullptr && n_columns >= 0) names = names_of(columns, n_columns);
    const std::vector<uint8_t> bytes = pop::read_local_file(path);
    auto ts = parquet_read(bytes.data(), static_cast<int64_t>(bytes.size()), names, start_pos, end_pos, s);
    export_tupleset(ts, out_schema, out, false, s);
  });
}

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
    const uint64_t launches0 = g_kernel_launches.load();
    auto fill_stats = [&](int64_t num_ops, int64_t messages) {
      if (stats == nullptr) return;
      stats->device_ns = 0;
      stats->kernel_launches = static_cast<int64_t>(g_kernel_launches.load() - launches0);
      stats->h2d_bytes = copy_counters().h2d - c0.h2d + copy_counters().in_place - c0.in_place;
      stats->d2h_bytes = copy_counters().d2h - c0.d2h;
      stats->num_ops = num_ops;
      stats->messages = messages;
      stats->elapsed_ns =
          std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    };
    // Replay of a captured plan: found before any parsing or import.
    const bool maybe_graph = std::strstr(plan_json, "\"cudaGraph\"") != nullptr;
    std::string key;
    if (maybe_graph) {
      key = plan_key(plan_json, n_tables, table_names, arrays);
      std::shared_ptr<CapturedPlan> cp;
      {
        std::lock_guard<std::mutex> lk(g_graph_mu);
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) cp = it->second;
      }
      int64_t device_ns = 0;
      if (cp && cp->capturable && replay_plan(*cp, result_to_host != 0, out_schema, out, s, &device_ns)) {
        fill_stats(cp->num_ops, cp->messages);
        if (stats != nullptr) stats->device_ns = device_ns;
        return;
      }
    }
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
    const bool deferred = plan.get_bool("deferredSizes", true);
    struct CopyModeGuard {
      explicit CopyModeGuard(int m) { set_host_copy_mode(m); }
      ~CopyModeGuard() { set_host_copy_mode(0); }
    } copy_mode(plan.get_str("hostCopy", "engine") == "sm" ? 1 : plan.get_str("hostCopy", "engine") == "zerocopy" ? 2 : 0);
    const bool use_graph = deferred && plan.get_bool("cudaGraph", false);
    TupleSetPtr result;
    pop::ExecStats xs;
    auto run_plain = [&](bool defer) {
      auto ex = pop::build_execution(plan, s);
      ex->setInputs(inputs);
      ex->setDeferred(defer);
      auto r = ex->execute();
      xs = ex->stats();
      return r;
    };
    auto run = [&]() {
      try {
        return run_plain(deferred);
      } catch (const pop::NeedsExactSizes&) {
        // A join met repeated build keys and overflowed its deferred
        // capacity: run the plan again with exact (synchronized) sizes.
        return run_plain(false);
      }
    };
    if (!use_graph) {
      result = run();
    } else {
      std::shared_ptr<CapturedPlan> cp;
      {
        std::lock_guard<std::mutex> lk(g_graph_mu);
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) cp = it->second;
      }
      // First call for these inputs: an ordinary run (which also measures the
      // memory the plan needs), then the capture; a replay that overflowed
      // lands here too and gets the exact re-run.
      const int64_t a0 = thread_alloc_bytes();
      int64_t f0[2][2], f1[2][2];
      thread_filled_bytes(f0);
      result = run();
      if (!cp) {
        const int64_t bytes = thread_alloc_bytes() - a0;
        thread_filled_bytes(f1);
        int64_t fills[2][2], spare = 0;
        for (int t = 0; t < 2; ++t)
          for (int k = 0; k < 2; ++k) {
            fills[t][k] = f1[t][k] - f0[t][k];
            spare += fills[t][k] / 4 + 4096;  // the arena also holds the fill regions' spare room
          }
        cp = capture_plan(plan, inputs, bytes + bytes / 4 + spare + (int64_t{1} << 20), fills);
        std::lock_guard<std::mutex> lk(g_graph_mu);
        g_graphs[key] = cp;
      }
    }
    export_tupleset(result, out_schema, out, result_to_host != 0, s);
    sync(s);
    fill_stats(xs.num_ops, xs.messages);
  });
}

int32_t gfpdb_graph_cache_clear(void) {
  return guarded([&] {
    {
      std::lock_guard<std::mutex> lk(g_graph_mu);
      g_graphs.clear();
    }
    clear_batches();
  });
}

int32_t gfpdb_star_batch(const char* spec_json, int32_t n_tables, const char* const* table_names,
                         const ArrowSchema* const* schemas, const ArrowDeviceArray* const* arrays, int32_t use_graph,
                         int32_t result_to_host, ArrowSchema* out_schema, ArrowDeviceArray* out,
                         gfpdb_exec_stats* stats, void* stream) {
  return guarded([&] {
    require(spec_json != nullptr && out_schema != nullptr && out != nullptr, "null argument");
    const auto t0 = std::chrono::steady_clock::now();
    ensure_device();
    cudaStream_t s = as_stream(stream);
    const CopyCounters c0 = copy_counters();
    const uint64_t launches0 = g_kernel_launches.load();
    const std::string key = std::string(use_graph ? "G|" : "P|") + plan_key(spec_json, n_tables, table_names, arrays);
    std::shared_ptr<BatchEntry> be = find_batch(key);
    if (!be) {
      json::Value spec;
      try {
        spec = json::parse(spec_json);
      } catch (const std::exception& e) {
        fail(GFPDB_EINVAL, e.what());
      }
      BatchInputs in = import_batch_inputs(n_tables, table_names, schemas, arrays, s);
      // pageable host memory cannot be copied from inside a CUDA graph
      be = make_batch(spec, in.tables, use_graph != 0 && !in.pageable, s, std::move(in.host_cols));
      remember_batch(key, be);
    }
    if (be->exec != nullptr) {
      GF_CUDA(cudaGraphLaunch(be->exec, s));
      count_launch(be->kernels);
    } else {
      be->batch.run(s);
    }
    DevStatus st;
    unsigned long long gathered[2] = {0, 0};
    GF_CUDA(cudaMemcpyAsync(&st, be->batch.status(), sizeof(st), cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaMemcpyAsync(gathered, be->batch.gathered(), sizeof(gathered), cudaMemcpyDeviceToHost, s));
    sync(s);
    // bytes from host memory: the copies, and the reads in place
    copy_counters().h2d += be->batch.host_bytes() + be->batch.in_place_bytes(gathered[0], gathered[1]);
    if (st.code == GFPDB_EINVAL && st.detail >= 100 && st.detail < 110)
      fail(GFPDB_EINVAL, "batched star query: dimension " + std::to_string(st.detail - 100) + " repeats a key");
    raise_device_status(st, "batched star query");
    export_tupleset(be->batch.result_view(), out_schema, out, result_to_host != 0, s);
    sync(s);
    if (stats != nullptr) {
      stats->kernel_launches = static_cast<int64_t>(g_kernel_launches.load() - launches0);
      stats->h2d_bytes = copy_counters().h2d - c0.h2d;
      stats->d2h_bytes = copy_counters().d2h - c0.d2h;
      stats->num_ops = 3;
      stats->messages = 0;
      stats->device_ns = 0;
      stats->elapsed_ns =
          std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

// ------------------------------------------------------- prepared batches

struct gfpdb_batch {
  std::shared_ptr<BatchEntry> be;
  TupleSetPtr result;       // the batch's device result view
  char* pinned = nullptr;   // status, row count and result columns, packed by the run
  int64_t pinned_bytes = 0;
  int64_t status_off = 0, count_off = 0, gathered_off = 0;
  std::vector<int64_t> col_off;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool in_flight = false;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;  // kernels per run
  ~gfpdb_batch() {
    if (in_flight && ev[1] != nullptr) (void)cudaEventSynchronize(ev[1]);
    for (auto e : ev)
      if (e) (void)cudaEventDestroy(e);
    be.reset();
    if (pinned) (void)cudaFreeHost(pinned);
  }
};

namespace {

// One run of a prepared batch on stream s: the stages, then the pack of its
// status, row count and result columns into page-locked memory.
void batch_run_and_pack(gfpdb_batch& b, const std::vector<CopySpan>& spans, cudaStream_t s) {
  b.be->batch.run(s);
  pack_spans(spans, b.pinned, s);
}

}  // namespace

int32_t gfpdb_batch_prepare(const char* spec_json, int32_t n_tables, const char* const* table_names,
                            const ArrowSchema* const* schemas, const ArrowDeviceArray* const* arrays,
                            gfpdb_batch** out) {
  return guarded([&] {
    require(spec_json != nullptr && out != nullptr, "null argument");
    ensure_device();
    cudaStream_t s = nullptr;
    json::Value spec;
    try {
      spec = json::parse(spec_json);
    } catch (const std::exception& e) {
      fail(GFPDB_EINVAL, e.what());
    }
    BatchInputs in = import_batch_inputs(n_tables, table_names, schemas, arrays, s);
    auto b = std::make_unique<gfpdb_batch>();
    b->be = make_batch(spec, in.tables, false, s, std::move(in.host_cols));
    b->result = b->be->batch.result_view();
    const TupleSet& r = *b->result;
    std::vector<CopySpan> spans;
    int64_t off = 0;
    auto add = [&](const void* src, int64_t bytes) {
      const int64_t o = off;
      spans.push_back(CopySpan{src, bytes, o});
      off += (bytes + 255) / 256 * 256;
      return o;
    };
    b->status_off = add(b->be->batch.status(), sizeof(DevStatus));
    b->gathered_off = add(b->be->batch.gathered(), 2 * sizeof(unsigned long long));
    b->count_off = add(r.rows_dev(), sizeof(int64_t));
    for (int i = 0; i < r.num_columns(); ++i) {
      const auto& c = r.column(i);
      b->col_off.push_back(add(c->data, r.num_rows() * dtype_width(c->type)));
    }
    b->pinned_bytes = off;
    GF_CUDA(cudaMallocHost(reinterpret_cast<void**>(&b->pinned), static_cast<size_t>(off)));
    std::memset(b->pinned, 0, static_cast<size_t>(off));
    GF_CUDA(cudaEventCreate(&b->ev[0]));
    GF_CUDA(cudaEventCreate(&b->ev[1]));
    if (!in.pageable) {
      // capture the run and the pack as one graph (pageable host memory
      // cannot be copied from inside a graph: such batches run uncaptured)
      cudaStream_t cs = nullptr;
      GF_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      const uint64_t k0 = g_kernel_launches.load();
      cudaGraph_t graph = nullptr;
      bool ok = true;
      GF_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      try {
        batch_run_and_pack(*b, spans, cs);
      } catch (const std::exception&) {
        ok = false;
      }
      if (cudaStreamEndCapture(cs, &graph) != cudaSuccess) ok = false;
      if (ok && cudaGraphInstantiate(&b->be->exec, graph, 0) != cudaSuccess) ok = false;
      if (graph) (void)cudaGraphDestroy(graph);
      (void)cudaGetLastError();
      (void)cudaStreamDestroy(cs);
      b->launches = static_cast<int64_t>(g_kernel_launches.load() - k0);
      if (!ok) fail(GFPDB_ECUDA, "capturing the batched star query failed");
    }
    b->be->spans = std::move(spans);
    *out = b.release();
  });
}

int32_t gfpdb_batch_launch(gfpdb_batch* b, void* stream) {
  return guarded([&] {
    require(b != nullptr, "null argument");
    if (b->in_flight) fail(GFPDB_EINVAL, "this prepared batch is already running; prepare a second copy");
    cudaStream_t s = as_stream(stream);
    GF_CUDA(cudaEventRecord(b->ev[0], s));
    const uint64_t k0 = g_kernel_launches.load();
    if (b->be->exec != nullptr) {
      GF_CUDA(cudaGraphLaunch(b->be->exec, s));
      count_launch(static_cast<uint64_t>(b->launches));
    } else {
      batch_run_and_pack(*b, b->be->spans, s);
      b->launches = static_cast<int64_t>(g_kernel_launches.load() - k0);
    }
    GF_CUDA(cudaEventRecord(b->ev[1], s));
    b->stream = s;
    b->in_flight = true;
  });
}

int32_t gfpdb_batch_wait(gfpdb_batch* b, gfpdb_exec_stats* stats, int64_t* n_rows) {
  return guarded([&] {
    require(b != nullptr && n_rows != nullptr, "null argument");
    if (!b->in_flight) fail(GFPDB_EINVAL, "the prepared batch has no run to wait for");
    const auto t0 = std::chrono::steady_clock::now();
    {
      struct Reset {
        gfpdb_batch* b;
        ~Reset() { b->in_flight = false; }
      } reset{b};
      // a batch is short: poll its end, then fall back to a blocking wait
      for (;;) {
        const cudaError_t q = cudaEventQuery(b->ev[1]);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) GF_CUDA(q);
        if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(2000)) {
          GF_CUDA(cudaEventSynchronize(b->ev[1]));
          break;
        }
      }
    }
    const DevStatus& st = *reinterpret_cast<const DevStatus*>(b->pinned + b->status_off);
    if (st.code == GFPDB_EINVAL && st.detail >= 100 && st.detail < 110)
      fail(GFPDB_EINVAL, "batched star query: dimension " + std::to_string(st.detail - 100) + " repeats a key");
    raise_device_status(st, "batched star query");
    const int64_t n = *reinterpret_cast<const int64_t*>(b->pinned + b->count_off);
    if (n < 0 || n > b->result->num_rows()) fail(GFPDB_EDEVICE, "batched star query produced an out-of-range row count");
    *n_rows = n;
    // bytes from host memory: the copies, and the reads in place
    const unsigned long long* g = reinterpret_cast<const unsigned long long*>(b->pinned + b->gathered_off);
    const int64_t h2d = b->be->batch.host_bytes() + b->be->batch.in_place_bytes(g[0], g[1]);
    copy_counters().h2d += h2d;
    copy_counters().d2h += b->pinned_bytes;
    if (stats != nullptr) {
      float ms = 0;
      GF_CUDA(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
      stats->device_ns = static_cast<int64_t>(static_cast<double>(ms) * 1e6);
      stats->kernel_launches = b->launches;
      stats->h2d_bytes = h2d;
      stats->d2h_bytes = b->pinned_bytes;
      stats->num_ops = 3;
      stats->messages = 0;
      stats->elapsed_ns =
          std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    }
  });
}

int32_t gfpdb_batch_run(gfpdb_batch* b, gfpdb_exec_stats* stats, void* stream, int64_t* n_rows) {
  const int32_t rc = gfpdb_batch_launch(b, stream);
  if (rc != GFPDB_OK) return rc;
  return gfpdb_batch_wait(b, stats, n_rows);
}

int32_t gfpdb_batch_layout(const gfpdb_batch* b, int32_t max_columns, int64_t* capacity, int32_t* n_columns,
                           char* names, int64_t names_capacity, const void** values) {
  return guarded([&] {
    require(b != nullptr && capacity != nullptr && n_columns != nullptr && names != nullptr && values != nullptr,
            "null argument");
    const TupleSet& r = *b->result;
    require(r.num_columns() <= max_columns, "more columns than max_columns");
    int64_t at = 0;
    auto put = [&](const char* str) {
      const int64_t len = static_cast<int64_t>(std::strlen(str)) + 1;
      require(at + len <= names_capacity, "column names exceed names_capacity");
      std::memcpy(names + at, str, static_cast<size_t>(len));
      at += len;
    };
    *capacity = r.num_rows();
    *n_columns = r.num_columns();
    for (int i = 0; i < r.num_columns(); ++i) {
      put(r.field(i).name.c_str());
      put(dtype_format(r.field(i).type));
      values[i] = b->pinned + b->col_off[static_cast<size_t>(i)];
    }
  });
}

void gfpdb_batch_free(gfpdb_batch* b) { delete b; }

int32_t gfpdb_plan_prepare(const char* plan_json, int32_t n_tables, const char* const* table_names,
                           const ArrowSchema* const* schemas, const ArrowDeviceArray* const* arrays,
                           gfpdb_prepared** out) {
  return guarded([&] {
    require(plan_json != nullptr && out != nullptr && n_tables >= 0, "null argument");
    require(n_tables == 0 || (table_names != nullptr && schemas != nullptr && arrays != nullptr), "null tables");
    json::Value plan;
    try {
      plan = json::parse(plan_json);
    } catch (const std::exception& e) {
      fail(GFPDB_EINVAL, e.what());
    }
    pop::validate_plan(plan);
    ensure_device();
    auto p = std::make_unique<gfpdb_prepared>();
    p->plan = plan_json;
    for (int32_t i = 0; i < n_tables; ++i) {
      require(table_names[i] != nullptr && schemas[i] != nullptr && arrays[i] != nullptr, "null table");
      p->names.push_back(table_names[i]);
      p->schemas.push_back(schemas[i]);
      p->arrays.push_back(arrays[i]);
    }
    for (auto& n : p->names) p->name_ptrs.push_back(n.c_str());
    p->graph = plan.get_bool("cudaGraph", false) && plan.get_bool("deferredSizes", true);
    if (p->graph) p->key = plan_key(plan_json, n_tables, table_names, arrays);
    *out = p.release();
  });
}

}  // extern "C"

namespace {

// An ordinary (non-replay) run of a prepared plan: its result is exported
// into the prepared plan's host buffers; afterwards the plan's capture, if
// one was made, is picked up for later launches.
void run_prepared_exact(gfpdb_prepared* p, gfpdb_exec_stats* stats) {
  p->release_result();
  const int32_t code = gfpdb_execute_plan(p->plan.c_str(), static_cast<int32_t>(p->names.size()),
                                          p->name_ptrs.data(), p->schemas.data(), p->arrays.data(), 1, &p->res_s,
                                          &p->res_a, stats, p->stream);
  if (code != GFPDB_OK) fail(code, std::string(gfpdb_last_error()));
  p->has_res = true;
  p->last_replay = false;
  ++p->generation;
  p->rows = p->res_a.array.length;
  p->find_capture();
}

}  // namespace

extern "C" {

int32_t gfpdb_prepared_launch(gfpdb_prepared* p, void* stream) {
  return guarded([&] {
    require(p != nullptr, "null argument");
    require(p->pending == gfpdb_prepared::kNone, "the prepared plan's last launch has not been waited for");
    p->t0 = std::chrono::steady_clock::now();
    p->stream = stream;
    p->find_capture();
    if (p->cp && p->cp->capturable) {
      replay_launch(*p->cp, as_stream(stream));
      p->pending = gfpdb_prepared::kReplay;
      return;
    }
    // the first runs (an ordinary run, then the capture) and plans without
    // a graph complete here
    run_prepared_exact(p, &p->done_stats);
    p->pending = gfpdb_prepared::kDone;
  });
}

int32_t gfpdb_prepared_wait(gfpdb_prepared* p, gfpdb_exec_stats* stats, int64_t* n_rows, int64_t* layout_generation) {
  return guarded([&] {
    require(p != nullptr && n_rows != nullptr && layout_generation != nullptr, "null argument");
    require(p->pending != gfpdb_prepared::kNone, "no launched run to wait for");
    const auto kind = p->pending;
    p->pending = gfpdb_prepared::kNone;
    if (kind == gfpdb_prepared::kReplay) {
      int64_t device_ns = 0, n = 0;
      if (replay_finish(*p->cp, as_stream(p->stream), &device_ns, &n)) {
        p->release_result();
        if (!p->last_replay) {
          ++p->generation;
          p->last_replay = true;
        }
        *n_rows = n;
        *layout_generation = p->generation;
        if (stats != nullptr) {
          // this replay's own figures (the process-wide counters would also
          // count another prepared plan's replay launched in between)
          stats->kernel_launches = static_cast<int64_t>(p->cp->kernels);
          stats->h2d_bytes = p->cp->h2d;
          stats->d2h_bytes = p->cp->pinned_bytes;
          stats->num_ops = p->cp->num_ops;
          stats->messages = p->cp->messages;
          stats->device_ns = device_ns;
          stats->elapsed_ns =
              std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - p->t0).count();
        }
        return;
      }
      // a deferred size overflowed: run once more with exact sizes
      run_prepared_exact(p, &p->done_stats);
    }
    if (stats != nullptr) *stats = p->done_stats;
    *n_rows = p->rows;
    *layout_generation = p->generation;
  });
}

int32_t gfpdb_prepared_run(gfpdb_prepared* p, gfpdb_exec_stats* stats, void* stream, int64_t* n_rows,
                           int64_t* layout_generation) {
  const int32_t code = gfpdb_prepared_launch(p, stream);
  if (code != GFPDB_OK) return code;
  return gfpdb_prepared_wait(p, stats, n_rows, layout_generation);
}

int32_t gfpdb_prepared_layout(const gfpdb_prepared* p, int32_t max_columns, int64_t* capacity, int32_t* n_columns,
                              char* names, int64_t names_capacity, const void** values, const void** offsets) {
  return guarded([&] {
    require(p != nullptr && capacity != nullptr && n_columns != nullptr && names != nullptr && values != nullptr &&
                offsets != nullptr,
            "null argument");
    int64_t at = 0;
    auto put = [&](const char* str) {
      const int64_t len = static_cast<int64_t>(std::strlen(str)) + 1;
      require(at + len <= names_capacity, "column names exceed names_capacity");
      std::memcpy(names + at, str, static_cast<size_t>(len));
      at += len;
    };
    if (p->last_replay) {
      const CapturedPlan& cp = *p->cp;
      const TupleSet& r = *cp.result;
      require(r.num_columns() <= max_columns, "more columns than max_columns");
      *capacity = r.num_rows();
      *n_columns = r.num_columns();
      for (int i = 0; i < r.num_columns(); ++i) {
        put(r.field(i).name.c_str());
        put(dtype_format(r.field(i).type));
        const auto& offs = cp.col_off[static_cast<size_t>(i)];
        if (r.field(i).type == DType::Utf8) {
          offsets[i] = cp.pinned + offs[0];
          values[i] = cp.pinned + offs[1];
        } else {
          values[i] = cp.pinned + offs[0];
          offsets[i] = nullptr;
        }
      }
      return;
    }
    require(p->has_res, "the prepared plan has not run");
    int64_t n = 0;
    int32_t device_type = 0;
    const int32_t code = gfpdb_result_layout(&p->res_s, &p->res_a, max_columns, &n, n_columns, &device_type, names,
                                             names_capacity, values, offsets);
    if (code != GFPDB_OK) fail(code, std::string(gfpdb_last_error()));
    *capacity = n;
  });
}

void gfpdb_prepared_free(gfpdb_prepared* p) {
  if (p == nullptr) return;
  // a replay launched and never waited for: let it finish before its
  // captured plan (scratch, result buffers) can go with this handle
  if (p->pending == gfpdb_prepared::kReplay && p->cp && p->cp->ev[1] != nullptr) {
    (void)cudaEventSynchronize(p->cp->ev[1]);
    p->cp->in_flight = false;
  }
  delete p;
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

int32_t gfpdb_plan_fuse(const char* plan_json, char* out_json, int64_t capacity, int64_t* needed) {
  return guarded([&] {
    require(plan_json != nullptr && needed != nullptr, "null argument");
    json::Value plan;
    try {
      plan = json::parse(plan_json);
    } catch (const std::exception& e) {
      fail(GFPDB_EINVAL, e.what());
    }
    const std::string out = json::dump(pop::fuse_pipelines(plan));
    *needed = static_cast<int64_t>(out.size()) + 1;
    if (out_json == nullptr || capacity < *needed) fail(GFPDB_EINVAL, "output buffer too small (see *needed)");
    std::memcpy(out_json, out.c_str(), out.size() + 1);
  });
}

int32_t gfpdb_plan_predicate_transfer(const char* spec_json, char* out_json, int64_t capacity, int64_t* needed) {
  return guarded([&] {
    require(spec_json != nullptr && needed != nullptr, "null argument");
    json::Value spec;
    try {
      spec = json::parse(spec_json);
    } catch (const std::exception& e) {
      fail(GFPDB_EINVAL, e.what());
    }
    const std::string out = pop::plan_predicate_transfer(spec);
    *needed = static_cast<int64_t>(out.size()) + 1;
    if (out_json == nullptr || capacity < *needed) fail(GFPDB_EINVAL, "output buffer too small (see *needed)");
    std::memcpy(out_json, out.c_str(), out.size() + 1);
  });
}

}  // extern "C"
