// Host-side entry points of the CUDA kernels (implemented in the .cu files
// of this directory). Everything here runs on the caller's stream.
#pragma once

#include <string>
#include <vector>

#include "../host/expr.h"
#include "../host/tupleset.h"

namespace gfpdb {

// ------------------------------------------------------------- gather.cu

// Concatenate utf8 columns into one, rebasing offsets.
ColumnPtr concat_utf8(const std::vector<const Column*>& parts, cudaStream_t s);

// Gather rows `idx[0..n)` of each source column into new columns. All
// fixed-width columns are gathered by one launch; utf8 columns take a length
// pass, a prefix sum and a byte copy.
struct GatherSpec {
  const Column* src;
  const int32_t* idx;        // row ids into src
  bool may_be_null = false;  // idx holds -1 for a null (the output gets a validity bitmap)
};

// Validity bitmaps ((n + 31) / 32 LSB-first words): bit i set when idx[i] >= 0;
// the concatenation of parts (a null bitmap pointer: every row valid).
BufferPtr validity_from_index(const int32_t* idx, int64_t n, cudaStream_t s);
BufferPtr validity_concat(const std::vector<std::pair<const uint32_t*, int64_t>>& parts, int64_t total,
                          cudaStream_t s);
// A column of n nulls.
ColumnPtr null_column(DType t, int64_t n, cudaStream_t s);
// With n_dev, n is a capacity and the kernels read the true count from the
// device (deferred sizes); utf8 columns need an exact n.
std::vector<ColumnPtr> gather_columns(const std::vector<GatherSpec>& specs, int64_t n, cudaStream_t s,
                                      const int64_t* n_dev = nullptr, BufferPtr n_owner = nullptr);

// Copy several device byte ranges into one contiguous device buffer (one
// CTA per range): bundles a captured plan's status blocks and result
// columns so a single copy brings them all to the host.
struct CopySpan {
  const void* src;
  int64_t bytes;
  int64_t dst_off;
};
void pack_spans(const std::vector<CopySpan>& spans, void* dst, cudaStream_t s);

// Fill up to two regions (16-byte aligned, sizes multiples of 16) with one
// byte value each, in one kernel launch.
struct FillSpan {
  void* dst;
  int64_t bytes;
  int32_t value;
  int32_t pad;
};
// max_blocks > 0 caps the grid (a fill with time to spare can run on a few
// SMs beside other work).
void fill_regions(const FillSpan* spans, int n, cudaStream_t s, int max_blocks = 0);

// Host-to-device copy of a scan's input: the copy engine (cudaMemcpyAsync),
// or, with host_copy_mode() == 1 and page-locked aligned sources of at least
// 1 MiB, a kernel whose loads read host memory over the chip-to-chip link.
void copy_h2d(void* dst, const void* src, int64_t bytes, cudaStream_t s);

// Exclusive prefix sum of n int32 values into n+1 int32 offsets (offsets[n] =
// total). Returns the total (synchronizes the stream).
int64_t exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s);
// The same without waiting: the total lands in st->value (st zeroed by the
// caller; a device error in st->code), so that several scans can share one
// synchronization.
void exclusive_scan_i32_async(const int32_t* in, int32_t* out, int64_t n, DevStatus* st, cudaStream_t s);

// ------------------------------------------------------------- bloom.cu

struct BloomFilterDev {
  BufferPtr blocks;     // num_blocks * 8 uint32 words
  int64_t num_blocks = 0;  // exact, or the capacity when nblocks_dev is set
  int64_t num_keys = 0;    // exact, or an upper bound when nblocks_dev is set
  int32_t num_hashes = 3;
  int32_t bits_per_key = 10;
  bool valid = true;
  // Set when the filter was sized on the device from deferred key counts.
  BufferPtr header;
  const uint64_t* nblocks_dev = nullptr;
  const int32_t* valid_dev = nullptr;
};
using BloomPtr = std::shared_ptr<const BloomFilterDev>;

// part_rows_dev[i] (optional) is the device row count of key_parts[i] when
// that part comes from a deferred TupleSet (its length is then a capacity).
BloomPtr bloom_build(const std::vector<const Column*>& key_parts, int32_t bits_per_key, int32_t num_hashes,
                     cudaStream_t s, const std::vector<const int64_t*>& part_rows_dev = {});
// Several filters over the same rows in one pass: key_parts[f] are filter
// f's key column in each part (every filter's parts the same rows), with its
// own bits per key and hash count; each filter is the one bloom_build makes
// from its parts.
constexpr int kBloomBuildManyMax = 8;
std::vector<BloomPtr> bloom_build_many(const std::vector<std::vector<const Column*>>& key_parts,
                                       const std::vector<int32_t>& bits_per_key, const std::vector<int32_t>& num_hashes,
                                       cudaStream_t s, const std::vector<const int64_t*>& part_rows_dev = {});

// ------------------------------------------------------------- select.cu

struct BloomProbe {
  BloomPtr bloom;
  std::string column;
};

struct SelectStats {
  int64_t rows_in = 0;
  int64_t rows_out = 0;
};

// Fused predicate + bloom probes + stable compaction + projection.
// `project` lists output column names (empty + all_columns = every column).
TupleSetPtr select_rows(const TupleSet& in, const CompiledPredicate* pred, const std::vector<BloomProbe>& probes,
                        const std::vector<std::string>& project, bool all_columns, cudaStream_t s,
                        SelectStats* stats = nullptr);

// ---------------------------------------------------------- hashjoin.cu

struct JoinTable {
  BufferPtr slots;          // capacity uint64 (tag << 32 | build row)
  BufferPtr status;         // build diagnostics: longest probe run, duplicate keys
  uint64_t capacity = 0;    // power of two
  TupleSetPtr build;        // concatenated build side
  int key_col = -1;
  DType key_type = DType::Int32;
  int64_t max_probe = 0;
  bool composite = false;   // keyed on the composite of several key columns (or of a utf8 key)
  BufferPtr matched;        // outer / semi joins: int32 per build row, 1 once a probe row matched it
};

// `filters` (at most kJoinBuildFiltersMax, integer keys only): bloom filters
// on the key column; a build row whose key fails one is left out of the
// table (it stays in t.build but no probe finds it), as if a bloom selection
// on the key had run before the build.
constexpr int kJoinBuildFiltersMax = 4;
void join_build_table(JoinTable& t, double load_factor, cudaStream_t s, const std::vector<BloomPtr>& filters = {});

// Probe `probe` on column `probe_key`; returns matching (probe row, build
// row) pairs as two device int32 arrays of length *n_out. With count_dev
// and deferred mode on, nothing waits: *n_out is the pairs' capacity (the
// probe's row capacity, enough when build keys are unique), *count_dev the
// device count, and an overflow is detected by the plan's final checks.
// Probe and materialise fixed-width output columns in one pass: probe
// columns `probe_cols` (indexes into probe) then build columns `build_cols`
// (indexes into t.build). In deferred mode (count_dev given) the row count
// stays on the device; an overflow (repeated build keys) is reported by the
// deferred checks.
std::vector<ColumnPtr> join_probe_materialize(const JoinTable& t, const TupleSet& probe, int probe_key,
                                              const std::vector<int>& probe_cols, const std::vector<int>& build_cols,
                                              int64_t* n_out, cudaStream_t s, BufferPtr* count_owner = nullptr,
                                              const int64_t** count_dev = nullptr);
void join_probe_pairs(const JoinTable& t, const TupleSet& probe, int probe_key, BufferPtr* probe_idx,
                      BufferPtr* build_idx, int64_t* n_out, cudaStream_t s, BufferPtr* count_owner = nullptr,
                      const int64_t** count_dev = nullptr);

// Outer and semi joins (exact probe batches). join_match: per probe row its
// output pairs into counts (matches, or 1 for an unmatched row when
// keep_unmatched; counts may be null), and 1 into matched[build row] for
// every build row matched (matched may be null).
void join_match(const JoinTable& t, const TupleSet& probe, int probe_key, int32_t* counts, bool keep_unmatched,
                int32_t* matched, cudaStream_t s);
// The (probe row, build row) pairs in probe-row order; with keep_unmatched
// a probe row without a match gives (row, -1).
void join_pairs_ordered(const JoinTable& t, const TupleSet& probe, int probe_key, bool keep_unmatched,
                        int32_t* matched, BufferPtr* pidx, BufferPtr* bidx, int64_t* n_out, cudaStream_t s);
// Row ids i < n with v[i] != 0 (nonzero) or v[i] == 0, in order.
BufferPtr rows_where(const int32_t* v, int64_t n, bool nonzero, int64_t* n_out, cudaStream_t s);

// A chain of inner joins probed in one pass: level l probes tables[l] with a
// key column taken from the input row (source 0) or from the build row that
// an earlier level k matched (source k + 1), and every combination of
// matches writes one output row. Fixed-width columns only. Output and
// capacity rules as join_probe_materialize (capacity: the input's rows).
struct ChainRef {
  int src;  // 0: the input; l + 1: tables[l]->build
  int col;  // column index in that TupleSet
};
constexpr int kJoinChainMax = 6;
std::vector<ColumnPtr> join_chain_materialize(const std::vector<const JoinTable*>& tables, const TupleSet& probe,
                                              const std::vector<ChainRef>& keys, const std::vector<ChainRef>& outs,
                                              int64_t* n_out, cudaStream_t s, BufferPtr* count_owner = nullptr,
                                              const int64_t** count_dev = nullptr);

// ------------------------------------------------------------- group.cu

// Column-name prefixes of a parallel AVG's intermediate sum and count
// (AggregatePrePFunction::AVG_INTERMEDIATE_*_COLUMN_PREFIX,
// fpdb-plan/include/fpdb/plan/prephysical/AggregatePrePFunction.h:25-26).
constexpr const char* kAvgIntermediateSum = "AVG_INTERMEDIATE_SUM_";
constexpr const char* kAvgIntermediateCount = "AVG_INTERMEDIATE_COUNT_";

struct GroupAggregate {
  AggFn fn;
  std::string name;
  ExprPtr expr;  // null for count(*)
  // filled when compiled against the first batch
  DType in_type = DType::Int64;
};

class GroupTable;
std::shared_ptr<GroupTable> group_table_create(const std::vector<std::string>& group_cols,
                                               const std::vector<GroupAggregate>& aggs, int64_t groups_hint);
void group_table_update(GroupTable& g, const TupleSet& batch, cudaStream_t s);
TupleSetPtr group_table_finalize(GroupTable& g, cudaStream_t s);

// --------------------------------------------------------- starbatch.cu

constexpr int kSBMaxDims = 8;
constexpr int kSBMaxQueries = 64;
constexpr int kSBMaxParts = 256;
constexpr int64_t kSBSmemBudget = 200 * 1024;       // staged query masks per SM
constexpr int64_t kSBSmemPerBlockMax = 200 * 1024;  // and per block
constexpr int64_t kSBSmemMaxDynamic = 220 * 1024;   // dynamic shared memory of one fact-stage block

// A batch of star queries over one partitioned fact table that differ only
// in their per-dimension filter ranges (lo <= filter column <= hi).
struct StarBatchSpec {
  struct Dim {
    std::string table, key, fact_key, filter;
  };
  struct Group {
    int dim;
    std::string column;
  };
  struct Agg {
    AggFn fn;  // AGG_SUM or AGG_COUNT_STAR
    std::string name;
    std::vector<std::string> columns;  // SUM of one fact column or of the product of two
  };
  std::vector<std::string> fact_tables;
  std::vector<Dim> dims;
  std::vector<Group> group;
  std::vector<Agg> aggs;
  std::vector<std::vector<std::pair<int64_t, int64_t>>> queries;  // [query][dim] = (lo, hi)
  std::vector<int> probe_order;  // dimension probe order; empty: shared-memory dimensions, then by size
  double load_factor = 0.5;      // join tables
  int items_per_thread = 2;      // fact rows per consumer thread per tile: 1, 2, 4 or 8
  int blocks_per_sm = 4;         // persistent CTAs per SM
  int stages = 3;                // foreign-key tiles in flight per CTA (2 to 8)
  bool direct = true;            // int32 keys in aligned columns: the direct fact pass
  int64_t groups_hint = 1024;    // upper bound on groups per query
};

// A column of a batched star input that lives in host memory: each run
// copies its bytes from `src` to the device copy at `dst` first (the dimension
// columns, then the fact partitions in groups, each group's fact pass starting
// as soon as its copies have landed).
struct StarBatchHostColumn {
  const void* dst;
  const void* src;
  int64_t bytes;
};

struct StarBatchState;

// Preallocates every buffer in prepare(); run() only clears and fills them,
// so it can be captured into a CUDA graph.
class StarBatch {
 public:
  StarBatch();
  ~StarBatch();
  StarBatchSpec& spec();
  std::vector<TupleSetPtr>& parts();       // fact partitions
  std::vector<TupleSetPtr>& dim_tables();  // one per spec().dims
  void prepare(cudaStream_t s);
  void run(cudaStream_t s);
  // (query_id, group columns..., aggregates...), row count on the device;
  // valid after run() until the next run().
  TupleSetPtr result_view() const;
  const DevStatus* status() const;
  int64_t fact_rows() const;
  // Replaces the query ranges (at most the prepared number of queries; the
  // remaining slots select nothing) without preparing again.
  void set_ranges(const std::vector<std::vector<std::pair<int64_t, int64_t>>>& q, cudaStream_t s);
  // Device array of kSBMaxQueries + 1 offsets: query q's rows of the result
  // are [off[q], off[q + 1]); valid after run().
  const unsigned long long* query_offsets() const;
  // Device copies of host-resident input columns, refreshed by every run
  // (set before prepare()); host_bytes() is what one run copies.
  void set_host_columns(std::vector<StarBatchHostColumn> cols);
  int64_t host_bytes() const;
  // Two device counters of the last run: rows that reached the lookups in
  // global memory, and rows that reached the group updates; and the bytes
  // such rows read in place from host memory (columns not copied).
  const unsigned long long* gathered() const;
  int64_t in_place_bytes(uint64_t ring_rows, uint64_t survivor_rows) const;

 private:
  std::unique_ptr<StarBatchState> st_;
};

// --------------------------------------------------------------- keys.cu

constexpr int kMaxKeyColumns = 8;
// Names of the columns multi-column joins add internally.
constexpr const char* kBuildKeyColumn = "__gfpdb_bkey";
constexpr const char* kProbeKeyColumn = "__gfpdb_pkey";
constexpr const char* kBuildKeyAlias = "__gfpdb_bk";
// `t` plus an int64 column `name` combining the hashes of the key columns
// (equal keys, equal values), and with a non-empty alias_prefix the key
// columns again under the names alias_prefix + "0", "1", ... (same buffers).
TupleSetPtr with_composite_key(const TupleSetPtr& t, const std::vector<std::string>& keys, const std::string& name,
                               const std::string& alias_prefix, cudaStream_t s);
bool is_internal_key_column(const std::string& name);

// ------------------------------------------------------------ parquet.cu

// Read the named columns (all when empty) of a Parquet file held in host
// memory; with start_pos <= end_pos only the row groups whose first column
// chunk starts in [start_pos, end_pos]. Synchronizes `s`.
TupleSetPtr parquet_read(const uint8_t* file, int64_t size, const std::vector<std::string>& names, int64_t start_pos,
                         int64_t end_pos, cudaStream_t s);

// ------------------------------------------------------------ shuffle.cu

constexpr int64_t kShuffleMaxSlots = 1024;
// The rows of a TupleSet in slot order (slot i = rows [offsets[i],
// offsets[i+1])), input order kept within a slot; a row's slot is a hash of
// its key columns. Synchronizes `s`.
struct ShuffleResult {
  TupleSetPtr rows;
  std::vector<int64_t> offsets;  // num_slots + 1
};
ShuffleResult shuffle_rows(const TupleSetPtr& in, const std::vector<std::string>& keys, int64_t num_slots,
                           cudaStream_t s);
// Rows [at, at + len) of an exact TupleSet, sharing its buffers.
TupleSetPtr slice_rows(const TupleSetPtr& ts, int64_t at, int64_t len);

// ------------------------------------------------------------ project.cu

constexpr int kMaxProjOut = 16;
constexpr int kMaxSortKeys = 4;

// Value expressions compiled against one input schema (ProjectPOp).
struct ProjectSpec {
  Program prog{};
  ColumnSlots slots;
  std::vector<Operand> ops;
  std::vector<DType> types;
  std::vector<std::string> names;
};
// One new column per expression, rows as the input's (deferred sizes kept).
TupleSetPtr project_columns(const ProjectSpec& spec, const TupleSet& in, cudaStream_t s);
// A utf8 column's values, or SUBSTRING(value FROM from FOR len) of each (n exact).
ColumnPtr substring_column(const Column& c, int64_t n, bool sub, int from, int len, cudaStream_t s);

struct SortKeySpec {
  std::string column;
  bool descending;
};
// The first k rows of the input in key order (ties by input row), at most
// 1,024; synchronizes when the input's size is deferred.
TupleSetPtr select_k(const TupleSetPtr& in, const std::vector<SortKeySpec>& keys, int64_t k, cudaStream_t s);

// --------------------------------------------------------------- csv.cu

struct CsvField {
  std::string name;
  DType type;
  bool decimal = false;  // text with a fractional part -> int64 scaled by 10^scale
  int32_t scale = 0;
};

TupleSetPtr csv_parse(const char* device_text, int64_t n_bytes, char delimiter, bool has_header,
                      const std::vector<CsvField>& fields, const std::vector<int>& emit, cudaStream_t s);

}  // namespace gfpdb
