#include "server.h"

#include <algorithm>
#include <chrono>
#include <cstring>

#include "../kernels/launch.h"
#include "batchspec.h"
#include "pop.h"

namespace gfpdb::serve {

namespace {

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

std::string cache_key(const std::string& t, const std::string& c) { return t + '\0' + c; }

int64_t column_bytes(const HostTable& ht, const HostColumn& c) {
  if (c.type == DType::Utf8) return (ht.rows + 1) * 4 + (ht.rows > 0 ? c.offsets[ht.rows] : 0);
  return ht.rows * dtype_width(c.type);
}

void release_arrow(ArrowSchema* s, ArrowDeviceArray* a) {
  if (a->array.release) a->array.release(&a->array);
  if (s->release) s->release(s);
}

// Columns (by table) that the scans of a plan read.
std::map<std::string, std::vector<std::string>> plan_inputs(const json::Value& plan,
                                                            const std::map<std::string, HostTable>& tables) {
  std::map<std::string, std::vector<std::string>> out;
  for (auto& o : plan.at("ops").array()) {
    const std::string type = o.at("type").str();
    if (type == "FileScanPOp") fail(GFPDB_EUNSUPPORTED, "served requests read registered tables, not files");
    if (type != "TableScanPOp" && type != "CsvScanPOp" && type != "ParquetScanPOp") continue;
    const std::string t = o.at("table").str();
    auto it = tables.find(t);
    if (it == tables.end()) fail(GFPDB_EINVAL, "request scans table '" + t + "' which is not registered");
    std::vector<std::string> cols;
    if (type == "CsvScanPOp" || type == "ParquetScanPOp") {  // the file's bytes, one value
      if (it->second.cols.empty()) fail(GFPDB_EINVAL, "table '" + t + "' has no columns");
      cols.push_back(it->second.cols[0].name);
    } else if (o.contains("columns")) {
      cols = o.str_list("columns");
    } else {
      for (auto& c : it->second.cols) cols.push_back(c.name);
    }
    auto& dst = out[t];
    for (auto& c : cols)
      if (std::find(dst.begin(), dst.end(), c) == dst.end()) dst.push_back(c);
  }
  return out;
}

}  // namespace

// ------------------------------------------------------------ column cache

ColumnCache::~ColumnCache() { clear(); }

void ColumnCache::clear() {
  std::lock_guard<std::mutex> lk(mu_);
  for (auto& kv : m_)
    if (kv.second.ready) (void)cudaEventDestroy(kv.second.ready);
  m_.clear();
  resident_ = 0;
}

bool ColumnCache::evict_for(int64_t bytes) {
  while (resident_ + bytes > cap_) {
    auto victim = m_.end();
    for (auto it = m_.begin(); it != m_.end(); ++it) {
      if (it->second.pins > 0) continue;
      if (victim == m_.end() || it->second.freq < victim->second.freq ||
          (it->second.freq == victim->second.freq && it->second.last < victim->second.last))
        victim = it;
    }
    if (victim == m_.end()) return false;
    resident_ -= victim->second.bytes;
    if (victim->second.ready) (void)cudaEventDestroy(victim->second.ready);
    m_.erase(victim);  // the device buffer is freed stream-ordered on its loading stream
    ++evictions_;
  }
  return true;
}

std::vector<ColumnPtr> ColumnCache::acquire_all(const std::vector<Want>& wants, cudaStream_t s, int64_t* misses,
                                                int64_t timeout_ms) {
  std::vector<std::string> keys;
  for (auto& w : wants) keys.push_back(cache_key(w.table, w.ht->cols.at(static_cast<size_t>(w.col)).name));
  std::unique_lock<std::mutex> lk(mu_);
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  for (;;) {
    // pin the hits so that making room cannot evict them
    std::vector<std::string> pinned;
    int64_t need = 0;
    std::vector<std::string> seen;
    for (size_t i = 0; i < wants.size(); ++i) {
      if (std::find(seen.begin(), seen.end(), keys[i]) != seen.end()) continue;
      seen.push_back(keys[i]);
      auto it = m_.find(keys[i]);
      if (it != m_.end()) {
        ++it->second.pins;
        pinned.push_back(keys[i]);
      } else {
        need += column_bytes(*wants[i].ht, wants[i].ht->cols[wants[i].col]);
      }
    }
    if (need > cap_) {
      for (auto& k : pinned) --m_[k].pins;
      fail(GFPDB_ENOMEM, "the columns of one request are larger than the column cache");
    }
    if (evict_for(need)) break;
    for (auto& k : pinned) --m_[k].pins;
    if (released_.wait_until(lk, deadline) == std::cv_status::timeout)
      fail(GFPDB_ENOMEM, "column cache full of columns in use (admission timed out)");
  }
  std::vector<ColumnPtr> out;
  std::vector<std::string> done;
  for (size_t i = 0; i < wants.size(); ++i) {
    const HostTable& ht = *wants[i].ht;
    const HostColumn& hc = ht.cols[wants[i].col];
    auto it = m_.find(keys[i]);
    const bool first = std::find(done.begin(), done.end(), keys[i]) == done.end();
    if (it != m_.end()) {
      Entry& e = it->second;
      if (first) {
        ++e.freq;
        e.last = ++tick_;
        ++hits_;
      } else {
        ++e.pins;  // a repeated want pins again (released once per want)
      }
      GF_CUDA(cudaStreamWaitEvent(s, e.ready, 0));
      out.push_back(e.col);
      done.push_back(keys[i]);
      continue;
    }
    Entry e;
    e.bytes = column_bytes(ht, hc);
    e.freq = 1;
    e.last = ++tick_;
    e.pins = 1;
    if (hc.type == DType::Utf8) {
      const int64_t nb = ht.rows > 0 ? hc.offsets[ht.rows] : 0;
      auto offs = make_buffer((ht.rows + 1) * 4, s);
      auto data = make_buffer(std::max<int64_t>(nb, 1), s);
      memcpy_h2d(offs->data(), hc.offsets, (ht.rows + 1) * 4, s);
      memcpy_h2d(data->data(), hc.values, nb, s);
      e.col = make_utf8_column(ht.rows, offs, data);
    } else {
      auto buf = make_buffer(std::max<int64_t>(e.bytes, 1), s);
      memcpy_h2d(buf->data(), hc.values, e.bytes, s);
      e.col = make_fixed_column(hc.type, ht.rows, buf);
    }
    GF_CUDA(cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming));
    GF_CUDA(cudaEventRecord(e.ready, s));
    resident_ += e.bytes;
    ++misses_;
    if (misses) ++*misses;
    out.push_back(e.col);
    m_.emplace(keys[i], std::move(e));
    done.push_back(keys[i]);
  }
  return out;
}

void ColumnCache::release(const std::string& table, const std::string& column) {
  {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = m_.find(cache_key(table, column));
    if (it != m_.end() && it->second.pins > 0) --it->second.pins;
  }
  released_.notify_all();
}

int64_t ColumnCache::resident() const {
  std::lock_guard<std::mutex> lk(mu_);
  return resident_;
}

void ColumnCache::counters(int64_t* hits, int64_t* misses, int64_t* evictions) const {
  std::lock_guard<std::mutex> lk(mu_);
  *hits = hits_;
  *misses = misses_;
  *evictions = evictions_;
}

// ------------------------------------------------------------------ server

struct Request {
  uint64_t ticket = 0;
  bool star = false;
  json::Value plan;
  std::map<std::string, std::vector<std::string>> inputs;  // plan: columns per scanned table
  std::string batch_key;
  json::Value batch;
  std::vector<std::pair<int64_t, int64_t>> ranges;
  int64_t est = 0;
  bool done = false;
  int32_t status = GFPDB_OK;
  std::string error;
  bool has_result = false;
  ArrowSchema schema{};
  ArrowDeviceArray array{};
  gfpdb_request_stats st{};
  ~Request() {
    if (has_result) release_arrow(&schema, &array);
  }
};

// A batch prepared for one shape of star request: its buffers, its captured
// graph, and the identity of the cached columns it was built over (it pins
// them only while it runs; if one was evicted and loaded again, it is
// prepared again).
struct PreparedBatch {
  StarBatch batch;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;
  std::vector<const Column*> ids;
  ~PreparedBatch() {
    if (exec) (void)cudaGraphExecDestroy(exec);
  }
};

Server::Server(Config c) : cfg_(c), cache_(c.cache_bytes) {
  if (cfg_.workers < 1 || cfg_.workers > 32) fail(GFPDB_EINVAL, "workers must be in [1, 32]");
  if (cfg_.max_batch < 1 || cfg_.max_batch > kSBMaxQueries) fail(GFPDB_EINVAL, "maxBatch must be in [1, 64]");
  if (cfg_.cache_bytes <= 0 || cfg_.hbm_budget < cfg_.cache_bytes)
    fail(GFPDB_EINVAL, "cacheBytes must be positive and at most hbmBudgetBytes");
  st_.hbm_budget = cfg_.hbm_budget;
  st_.cache_capacity = cfg_.cache_bytes;
  GF_CUDA(cudaSetDevice(cfg_.device));
  for (int w = 0; w < cfg_.workers; ++w) {
    cudaStream_t s = nullptr;
    GF_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    streams_.push_back(s);
  }
  for (int w = 0; w < cfg_.workers; ++w) workers_.emplace_back([this, w] { worker_main(w); });
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  work_cv_.notify_all();
  admit_cv_.notify_all();
  for (auto& t : workers_) t.join();
  requests_.clear();
  cache_.clear();
  for (auto s : streams_) {
    (void)cudaStreamSynchronize(s);
    (void)cudaStreamDestroy(s);
  }
}

void Server::register_table(const std::string& name, HostTable t) {
  std::lock_guard<std::mutex> lk(mu_);
  if (tables_.count(name)) fail(GFPDB_EINVAL, "table '" + name + "' is already registered");
  tables_.emplace(name, std::move(t));
}

int64_t Server::estimate(const Request& r) const {
  // Working memory besides the cached inputs: plans materialise at most
  // about twice their inputs; a batched run's tables are a few hundred MB.
  if (r.star) return int64_t{512} << 20;
  int64_t in = 0;
  for (auto& kv : r.inputs) {
    const HostTable& ht = tables_.at(kv.first);
    for (auto& c : kv.second)
      for (auto& hc : ht.cols)
        if (hc.name == c) in += column_bytes(ht, hc);
  }
  return 2 * in + (int64_t{64} << 20);
}

uint64_t Server::submit(const std::string& text) {
  json::Value req;
  try {
    req = json::parse(text);
  } catch (const std::exception& e) {
    fail(GFPDB_EINVAL, e.what());
  }
  auto r = std::make_shared<Request>();
  const std::string kind = req.get_str("kind", "plan");
  std::lock_guard<std::mutex> lk(mu_);
  if (stop_) fail(GFPDB_EINVAL, "server is stopping");
  if (kind == "plan") {
    r->plan = req.at("plan");
    pop::validate_plan(r->plan);
    r->inputs = plan_inputs(r->plan, tables_);
  } else if (kind == "star") {
    r->star = true;
    r->batch = req.at("batch");
    r->batch_key = json_dump(r->batch);
    const size_t nd = r->batch.at("dimensions").array().size();
    for (auto& rg : req.at("ranges").array())
      r->ranges.emplace_back(rg.array().at(0).integer(), rg.array().at(1).integer());
    if (r->ranges.size() != nd) fail(GFPDB_EINVAL, "a star request needs one range per dimension");
    for (auto& t : r->batch.str_list("factTables"))
      if (!tables_.count(t)) fail(GFPDB_EINVAL, "request names table '" + t + "' which is not registered");
    for (auto& d : r->batch.at("dimensions").array())
      if (!tables_.count(d.at("table").str()))
        fail(GFPDB_EINVAL, "request names table '" + d.at("table").str() + "' which is not registered");
  } else {
    fail(GFPDB_EINVAL, "request kind must be \"plan\" or \"star\"");
  }
  r->est = estimate(*r);
  r->ticket = next_ticket_++;
  r->st.submit_ns = now_ns();
  requests_[r->ticket] = r;
  queue_.push_back(r);
  ++st_.submitted;
  work_cv_.notify_one();
  return r->ticket;
}

int32_t Server::wait(uint64_t ticket, int64_t timeout_ms, ArrowSchema* schema, ArrowDeviceArray* array,
                     gfpdb_request_stats* st) {
  std::unique_lock<std::mutex> lk(mu_);
  auto it = requests_.find(ticket);
  if (it == requests_.end()) fail(GFPDB_EINVAL, "unknown ticket " + std::to_string(ticket));
  std::shared_ptr<Request> r = it->second;
  auto ready = [&] { return r->done; };
  if (timeout_ms < 0) {
    done_cv_.wait(lk, ready);
  } else if (!done_cv_.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    return GFPDB_ETIMEDOUT;
  }
  requests_.erase(ticket);
  if (st) {
    *st = r->st;
    st->status = r->status;
  }
  if (r->status != GFPDB_OK) fail(r->status, r->error);
  if (schema && array && r->has_result) {
    *schema = r->schema;
    *array = r->array;
    r->has_result = false;  // the caller owns it now
  }
  return GFPDB_OK;
}

void Server::stats(gfpdb_server_stats* out) {
  std::lock_guard<std::mutex> lk(mu_);
  cache_.counters(&st_.cache_hits, &st_.cache_misses, &st_.cache_evictions);
  st_.cache_bytes = cache_.resident();
  st_.reserved_bytes = reserved_;
  *out = st_;
}

std::map<std::string, TupleSetPtr> Server::cached_tables(const std::map<std::string, std::vector<std::string>>& need,
                                                         cudaStream_t s,
                                                         std::vector<std::pair<std::string, std::string>>* pins,
                                                         int64_t* misses) {
  std::vector<ColumnCache::Want> wants;
  std::vector<std::pair<std::string, std::string>> names;
  {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& kv : need) {
      const HostTable& ht = tables_.at(kv.first);
      for (auto& name : kv.second) {
        int ci = -1;
        for (size_t i = 0; i < ht.cols.size(); ++i)
          if (ht.cols[i].name == name) ci = static_cast<int>(i);
        if (ci < 0) fail(GFPDB_EINVAL, "table '" + kv.first + "' has no column '" + name + "'");
        wants.push_back(ColumnCache::Want{kv.first, &ht, ci});
        names.emplace_back(kv.first, name);
      }
    }
  }
  std::vector<ColumnPtr> cols = cache_.acquire_all(wants, s, misses, cfg_.admission_timeout_ms);
  for (auto& n : names) pins->push_back(n);
  std::map<std::string, TupleSetPtr> out;
  size_t k = 0;
  for (auto& kv : need) {
    std::vector<Field> fields;
    std::vector<ColumnPtr> tc;
    for (auto& name : kv.second) {
      fields.push_back(Field{name, cols[k]->type});
      tc.push_back(cols[k]);
      ++k;
    }
    out[kv.first] = TupleSet::make(std::move(fields), std::move(tc), wants[k - 1].ht->rows);
  }
  return out;
}

void Server::unpin(const std::vector<std::pair<std::string, std::string>>& pins) {
  for (auto& p : pins) cache_.release(p.first, p.second);
}

void Server::run_plan(cudaStream_t s, Request& r) {
  std::vector<std::pair<std::string, std::string>> pins;
  struct Unpin {
    Server* sv;
    std::vector<std::pair<std::string, std::string>>* p;
    ~Unpin() { sv->unpin(*p); }
  } unpin_guard{this, &pins};
  int64_t misses = 0;
  std::map<std::string, pop::InputTable> inputs;
  for (auto& kv : cached_tables(r.inputs, s, &pins, &misses)) inputs[kv.first].device = kv.second;
  json::Value plan = r.plan;
  if (!plan.contains("streams")) {
    json::Value n;
    n.kind = json::Value::Number;
    n.is_integer = true;
    n.i = cfg_.plan_streams;
    plan.o.emplace_back("streams", n);
  }
  TupleSetPtr res;
  try {
    auto ex = pop::build_execution(plan, s);
    ex->setInputs(inputs);
    res = ex->execute();
  } catch (const pop::NeedsExactSizes&) {
    auto ex = pop::build_execution(plan, s);
    ex->setDeferred(false);
    ex->setInputs(inputs);
    res = ex->execute();
  }
  export_tupleset(res, &r.schema, &r.array, true, s);
  r.has_result = true;
  r.st.cache_misses = misses;
}

void Server::run_star(cudaStream_t s, std::vector<std::shared_ptr<Request>>& group,
                      std::map<std::string, std::unique_ptr<PreparedBatch>>& prepared, std::deque<std::string>& lru) {
  const std::string& key = group[0]->batch_key;
  StarBatchSpec shape;
  parse_star_batch_spec(group[0]->batch, shape);
  std::map<std::string, std::vector<std::string>> need;
  for (auto& tc : star_batch_columns(shape)) need[tc.first].push_back(tc.second);
  std::vector<std::pair<std::string, std::string>> pins;
  struct Unpin {
    Server* sv;
    std::vector<std::pair<std::string, std::string>>* p;
    ~Unpin() { sv->unpin(*p); }
  } unpin_guard{this, &pins};
  int64_t misses = 0;
  auto tabs = cached_tables(need, s, &pins, &misses);
  std::vector<const Column*> ids;
  for (auto& kv : tabs)
    for (int c = 0; c < kv.second->num_columns(); ++c) ids.push_back(kv.second->column(c).get());
  auto it = prepared.find(key);
  if (it == prepared.end() || it->second->ids != ids) {
    auto pb = std::make_unique<PreparedBatch>();
    StarBatchSpec& sp = pb->batch.spec();
    sp = shape;
    sp.queries.assign(static_cast<size_t>(cfg_.max_batch),
                      std::vector<std::pair<int64_t, int64_t>>(sp.dims.size(), {1, 0}));
    for (auto& t : sp.fact_tables) pb->batch.parts().push_back(tabs.at(t));
    for (auto& d : sp.dims) pb->batch.dim_tables().push_back(tabs.at(d.table));
    pb->batch.prepare(s);
    if (cfg_.graphs) pb->exec = capture_star_batch(pb->batch, &pb->kernels);
    pb->ids = ids;
    if (it != prepared.end()) {
      it->second = std::move(pb);
      lru.erase(std::find(lru.begin(), lru.end(), key));
    } else {
      it = prepared.emplace(key, std::move(pb)).first;
    }
    lru.push_back(key);
    while (lru.size() > 4) {  // prepared batches kept per worker
      prepared.erase(lru.front());
      lru.pop_front();
    }
    it = prepared.find(key);
  } else {
    lru.erase(std::find(lru.begin(), lru.end(), key));
    lru.push_back(key);
  }
  PreparedBatch& pb = *it->second;
  std::vector<std::vector<std::pair<int64_t, int64_t>>> q;
  for (auto& r : group) q.push_back(r->ranges);
  pb.batch.set_ranges(q, s);
  if (pb.exec) {
    GF_CUDA(cudaGraphLaunch(pb.exec, s));
    count_launch(pb.kernels);
  } else {
    pb.batch.run(s);
  }
  DevStatus st;
  unsigned long long off[kSBMaxQueries + 1];
  GF_CUDA(cudaMemcpyAsync(&st, pb.batch.status(), sizeof(st), cudaMemcpyDeviceToHost, s));
  GF_CUDA(cudaMemcpyAsync(off, pb.batch.query_offsets(), sizeof(off), cudaMemcpyDeviceToHost, s));
  sync(s);
  if (st.code == GFPDB_EINVAL && st.detail >= 100 && st.detail < 110)
    fail(GFPDB_EINVAL, "batched star query: dimension " + std::to_string(st.detail - 100) + " repeats a key");
  raise_device_status(st, "batched star query");
  // one copy of every result row, then each request's slice
  TupleSetPtr view = pb.batch.result_view();
  const int64_t total = static_cast<int64_t>(off[kSBMaxQueries]);
  std::vector<std::vector<char>> host(static_cast<size_t>(view->num_columns()));
  for (int c = 1; c < view->num_columns(); ++c) {
    const int w = dtype_width(view->column(c)->type);
    host[c].resize(static_cast<size_t>(std::max<int64_t>(total, 1) * w));
    if (total > 0)
      GF_CUDA(cudaMemcpyAsync(host[c].data(), view->column(c)->data, total * w, cudaMemcpyDeviceToHost, s));
  }
  sync(s);
  std::vector<Field> fields(view->fields().begin() + 1, view->fields().end());
  for (size_t i = 0; i < group.size(); ++i) {
    const int64_t o = static_cast<int64_t>(off[i]);
    const int64_t n = static_cast<int64_t>(off[i + 1]) - o;
    std::vector<std::vector<const void*>> bufs;
    for (int c = 1; c < view->num_columns(); ++c)
      bufs.push_back({host[c].data() + o * dtype_width(view->column(c)->type)});
    export_host_columns(fields, n, bufs, &group[i]->schema, &group[i]->array);
    group[i]->has_result = true;
    group[i]->st.kernel_launches = static_cast<int64_t>(pb.kernels) / static_cast<int64_t>(group.size());
    group[i]->st.cache_misses = misses;
  }
}

void Server::run_group(int, cudaStream_t s, std::vector<std::shared_ptr<Request>>& group,
                       std::map<std::string, std::unique_ptr<PreparedBatch>>& prepared, std::deque<std::string>& lru) {
  try {
    if (group[0]->star) {
      run_star(s, group, prepared, lru);
    } else {
      const uint64_t l0 = thread_kernel_launches();
      run_plan(s, *group[0]);
      group[0]->st.kernel_launches = static_cast<int64_t>(thread_kernel_launches() - l0);
    }
  } catch (const Error& e) {
    (void)cudaStreamSynchronize(s);
    for (auto& r : group) {
      r->status = e.code();
      r->error = e.what();
    }
  } catch (const std::exception& e) {
    (void)cudaStreamSynchronize(s);
    for (auto& r : group) {
      r->status = GFPDB_EINVAL;
      r->error = e.what();
    }
  }
}

void Server::worker_main(int w) {
  cudaStream_t s = streams_[static_cast<size_t>(w)];
  bool ok = cudaSetDevice(cfg_.device) == cudaSuccess;
  try {
    if (ok) ensure_device();
  } catch (...) {
    ok = false;
  }
  std::map<std::string, std::unique_ptr<PreparedBatch>> prepared;
  std::deque<std::string> lru;
  const int64_t work_budget = std::max<int64_t>(0, cfg_.hbm_budget - cfg_.cache_bytes);
  for (;;) {
    std::vector<std::shared_ptr<Request>> group;
    int64_t est = 0;
    {
      std::unique_lock<std::mutex> lk(mu_);
      work_cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
      if (queue_.empty()) break;  // stopping
      group.push_back(queue_.front());
      queue_.pop_front();
      if (group[0]->star && cfg_.batching) {
        for (auto it = queue_.begin(); it != queue_.end() && static_cast<int>(group.size()) < cfg_.max_batch;) {
          if ((*it)->star && (*it)->batch_key == group[0]->batch_key) {
            group.push_back(*it);
            it = queue_.erase(it);
          } else {
            ++it;
          }
        }
      }
      for (auto& r : group) est += r->est;
      // admission: the working-memory estimate must fit next to the requests
      // already running (a request alone is always admitted)
      const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(cfg_.admission_timeout_ms);
      bool admitted = true;
      if (inflight_ > 0 && reserved_ + est > work_budget) ++st_.admission_waits;
      while (!stop_ && inflight_ > 0 && reserved_ + est > work_budget) {
        if (admit_cv_.wait_until(lk, deadline) == std::cv_status::timeout) {
          admitted = false;
          break;
        }
      }
      if (!admitted || !ok) {
        for (auto& r : group) {
          r->status = ok ? GFPDB_ENOMEM : GFPDB_ECUDA;
          r->error = ok ? "request did not fit the HBM budget before the admission timeout"
                        : "server worker could not set up its device";
          r->done = true;
          r->st.end_ns = now_ns();
          ++st_.failed;
        }
        done_cv_.notify_all();
        continue;
      }
      reserved_ += est;
      ++inflight_;
      const int64_t t = now_ns();
      for (auto& r : group) {
        r->st.start_ns = t;
        r->st.worker = w;
        r->st.batch_size = static_cast<int32_t>(group.size());
      }
      if (group.size() > 1 || group[0]->star) {
        ++st_.batches;
        st_.batched_requests += static_cast<int64_t>(group.size());
      }
    }
    run_group(w, s, group, prepared, lru);
    {
      std::lock_guard<std::mutex> lk(mu_);
      reserved_ -= est;
      --inflight_;
      const int64_t t = now_ns();
      for (auto& r : group) {
        r->st.end_ns = t;
        r->done = true;
        if (r->status == GFPDB_OK) ++st_.completed;
        else ++st_.failed;
      }
    }
    admit_cv_.notify_all();
    done_cv_.notify_all();
  }
  prepared.clear();
  (void)cudaStreamSynchronize(s);
}

}  // namespace gfpdb::serve
