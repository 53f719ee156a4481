// Request server: the serving form of the hot path on one GPU.
//
// The reference serves queries through its client/server front end and keeps
// hot segments in fpdb-cache's SegmentCache (fpdb-cache/src/SegmentCache.cpp:21-75,
// LFU policy fpdb-cache/src/policy/LFUCachingPolicy.cpp), loaded by CacheLoadPOp
// (fpdb-executor/src/physical/cache/CacheLoadPOp.cpp:64-261). Here:
//   - tables are registered once as host-memory Arrow arrays; their columns
//     are loaded into an HBM-resident column cache on first use and evicted
//     least-frequently-used first (ties: least recently used) when the cache
//     is over its byte capacity, never while a request in flight uses them;
//   - worker threads, each with its own CUDA stream, take requests from one
//     queue, so requests overlap on the device;
//   - a request starts only when its working-memory estimate fits the HBM
//     budget next to the requests already running (admission);
//   - continuous batching: when a worker frees up, it takes the oldest
//     request and, if that is a batchable star query, every queued star query
//     of the same shape (up to the batch capacity) into one shared run of
//     the batched star engine; requests that arrive meanwhile join the next
//     batch. Every request's result is its own rows, identical to running it
//     alone.
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../../include/gfpdb.h"
#include "json.h"
#include "tupleset.h"

namespace gfpdb::serve {

struct Config {
  int device = 0;
  int workers = 4;
  int64_t hbm_budget = int64_t{120} << 30;   // cache plus working memory
  int64_t cache_bytes = int64_t{100} << 30;  // column cache capacity
  int max_batch = 64;
  bool batching = true;
  int plan_streams = 2;  // streams per plan execution (unless the plan says)
  bool graphs = true;    // batched runs replay a captured graph
  int64_t admission_timeout_ms = 120000;
};

// A registered table: host column buffers the caller keeps alive while the
// server exists.
struct HostColumn {
  std::string name;
  DType type = DType::Int32;
  const void* values = nullptr;      // fixed width: first value; utf8: bytes base
  const int32_t* offsets = nullptr;  // utf8: rows + 1 offsets into `values`
};
struct HostTable {
  std::vector<HostColumn> cols;
  int64_t rows = 0;
};

class ColumnCache {
 public:
  explicit ColumnCache(int64_t capacity) : cap_(capacity) {}
  ~ColumnCache();
  struct Want {
    std::string table;
    const HostTable* ht;
    int col;
  };
  // The device columns of `wants`, all pinned until release(): hits first,
  // then room is made by evicting unpinned columns (least frequently used,
  // then least recently used) and the misses are loaded on `s`. All or
  // nothing: while there is no room the caller waits, holding no pins, until
  // other requests release theirs; GFPDB_ENOMEM after timeout_ms or when the
  // columns alone exceed the capacity.
  std::vector<ColumnPtr> acquire_all(const std::vector<Want>& wants, cudaStream_t s, int64_t* misses,
                                     int64_t timeout_ms);
  void release(const std::string& table, const std::string& column);
  int64_t resident() const;
  int64_t capacity() const { return cap_; }
  // Drops every column (their buffers are freed on the streams that loaded
  // them, so call it while those streams exist).
  void clear();
  void counters(int64_t* hits, int64_t* misses, int64_t* evictions) const;

 private:
  struct Entry {
    ColumnPtr col;
    int64_t bytes = 0;
    uint64_t freq = 0;
    uint64_t last = 0;
    int pins = 0;
    cudaEvent_t ready = nullptr;  // load completion, on the loading stream
  };
  bool evict_for(int64_t bytes);  // mu_ held
  int64_t cap_;
  mutable std::mutex mu_;
  std::condition_variable released_;
  std::map<std::string, Entry> m_;
  int64_t resident_ = 0;
  uint64_t tick_ = 0;
  int64_t hits_ = 0, misses_ = 0, evictions_ = 0;
};

struct Request;
struct PreparedBatch;

class Server {
 public:
  explicit Server(Config c);
  ~Server();
  void register_table(const std::string& name, HostTable t);
  uint64_t submit(const std::string& request_json);
  // GFPDB_OK with the result moved out (schema/array may be null to drop it),
  // GFPDB_ETIMEDOUT when not finished within timeout_ms (< 0: wait forever);
  // a failed request throws its error.
  int32_t wait(uint64_t ticket, int64_t timeout_ms, ArrowSchema* schema, ArrowDeviceArray* array,
               gfpdb_request_stats* st);
  void stats(gfpdb_server_stats* out);

 private:
  void worker_main(int w);
  void run_group(int w, cudaStream_t s, std::vector<std::shared_ptr<Request>>& group,
                 std::map<std::string, std::unique_ptr<PreparedBatch>>& prepared, std::deque<std::string>& lru);
  void run_plan(cudaStream_t s, Request& r);
  void run_star(cudaStream_t s, std::vector<std::shared_ptr<Request>>& group,
                std::map<std::string, std::unique_ptr<PreparedBatch>>& prepared, std::deque<std::string>& lru);
  // Device TupleSets of the given columns of each table, pinned in the cache
  // (appended to *pins) until unpin().
  std::map<std::string, TupleSetPtr> cached_tables(const std::map<std::string, std::vector<std::string>>& need,
                                                   cudaStream_t s, std::vector<std::pair<std::string, std::string>>* pins,
                                                   int64_t* misses);
  void unpin(const std::vector<std::pair<std::string, std::string>>& pins);
  int64_t estimate(const Request& r) const;

  Config cfg_;
  ColumnCache cache_;
  std::mutex mu_;
  std::condition_variable work_cv_, done_cv_, admit_cv_;
  std::map<std::string, HostTable> tables_;
  std::deque<std::shared_ptr<Request>> queue_;
  std::map<uint64_t, std::shared_ptr<Request>> requests_;
  std::vector<std::thread> workers_;
  std::vector<cudaStream_t> streams_;  // one per worker; outlive the cached columns loaded on them
  bool stop_ = false;
  uint64_t next_ticket_ = 1;
  int64_t reserved_ = 0;
  int inflight_ = 0;
  gfpdb_server_stats st_{};
};

}  // namespace gfpdb::serve
