// Composite keys of several columns: the multi-column join and bloom keys of
// the reference's operators (HashJoinPredicate's column lists,
// fpdb-executor/include/fpdb/executor/physical/join/hashjoin/HashJoinPredicate.h:25-26;
// BloomFilterCreatePOp's and BloomFilterUseKernel::filter's column lists,
// fpdb-executor/src/physical/bloomfilter/BloomFilterCreatePOp.cpp:17-22,
// BloomFilterUseKernel.cpp:12-15).
//
// A key of k columns becomes one int64 column holding a 64-bit combination
// of the columns' hashes (integers by value, so int32 and int64 columns with
// equal values agree; utf8 by bytes), which the single-column bloom and join
// kernels then take as their key. Equal keys always get equal composites; a
// join on composites may in principle also pair unequal keys whose
// composites collide, so the join compares the key columns themselves
// afterwards (a selection on the joined rows), which makes it exact.
#include <cstring>

#include "common.cuh"
#include "launch.h"

namespace gfpdb {
namespace {

struct KeyHashParams {
  DevCol cols[kMaxKeyColumns];
  int32_t n_cols;
  int32_t pad;
  int64_t n;
  const int64_t* n_dev;
  int64_t* out;
};

__global__ void __launch_bounds__(256) key_hash_kernel(const __grid_constant__ KeyHashParams p) {
  int64_t n = p.n;
  if (p.n_dev != nullptr && *p.n_dev < n) n = *p.n_dev;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride)
    p.out[row] = static_cast<int64_t>(row_key_hash(p.cols, p.n_cols, row));
}

}  // namespace

TupleSetPtr with_composite_key(const TupleSetPtr& t, const std::vector<std::string>& keys, const std::string& name,
                               const std::string& alias_prefix, cudaStream_t s) {
  if (keys.empty() || keys.size() > static_cast<size_t>(kMaxKeyColumns))
    fail(GFPDB_EUNSUPPORTED, "a key has 1 to 8 columns");
  KeyHashParams p;
  std::memset(&p, 0, sizeof(p));
  std::vector<Field> fields = t->fields();
  std::vector<ColumnPtr> cols;
  for (int i = 0; i < t->num_columns(); ++i) cols.push_back(t->column(i));
  for (size_t i = 0; i < keys.size(); ++i) {
    const int ci = t->require_column(keys[i]);
    const auto& c = t->column(ci);
    if (c->type == DType::Float64) fail(GFPDB_EUNSUPPORTED, "float64 key column '" + keys[i] + "'");
    p.cols[i] = DevCol{c->data, c->offsets, static_cast<int32_t>(c->type), 0};
    if (!alias_prefix.empty()) {
      // the key column again under another name (same buffers): both sides'
      // keys stay in a join's output for the comparison, whatever their names
      fields.push_back(Field{alias_prefix + std::to_string(i), c->type});
      cols.push_back(c);
    }
  }
  p.n_cols = static_cast<int32_t>(keys.size());
  const int64_t cap = t->num_rows();
  auto buf = make_buffer(cap * 8, s);
  p.n = cap;
  p.n_dev = t->rows_dev();
  p.out = buf->as<int64_t>();
  if (cap > 0) {
    int64_t blocks = (cap + 255) / 256;
    const int64_t most = static_cast<int64_t>(num_sms()) * 8;
    if (blocks > most) blocks = most;
    ProfScope prof("key_hash_kernel", s);
    key_hash_kernel<<<static_cast<int>(blocks), 256, 0, s>>>(p);
    after_launch("key_hash_kernel");
    prof.stop(static_cast<double>(cap) * (8.0 + 4.0 * p.n_cols));
  }
  fields.push_back(Field{name, DType::Int64});
  cols.push_back(make_fixed_column(DType::Int64, cap, buf));
  if (t->exact()) return TupleSet::make(std::move(fields), std::move(cols), cap);
  return TupleSet::make_deferred(std::move(fields), std::move(cols), cap, t->rows_owner(), t->rows_dev());
}

bool is_internal_key_column(const std::string& name) { return name.rfind("__gfpdb_", 0) == 0; }

}  // namespace gfpdb
