// Expression projection (ProjectPOp) and top-k selection (LimitSortPOp).
//
// Projection evaluates up to kMaxProjOut value expressions per row (columns,
// literals, postfix arithmetic with Gandiva's typing, compiled by
// host/expr.cpp) into new columns, one pass over the rows.
//
// Top-k keeps the k first rows in the order of one to kMaxSortKeys keys,
// each ascending or descending, as arrow::compute::SelectKUnstable +
// arrow::compute::Take do for the reference's LimitSortPOp
// (fpdb-executor/src/physical/limitsort/LimitSortPOp.cpp:97-135). Rounds of
// block sorts: each block sorts 2048 row ids (bitonic network in shared
// memory, every id carrying a 64-bit order-preserving prefix of its first
// key so most comparisons touch no column) and keeps its first k; the kept
// ids of all blocks are the next round's input, until one block remains.
// Ties are broken by row id, so the result is deterministic: the first k
// rows of a stable sort.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "eval.cuh"
#include "launch.h"

namespace gfpdb {
namespace {

struct ProjectParams {
  Program prog;
  DevCol cols[kMaxCols];
  Operand ops[kMaxProjOut];
  void* out[kMaxProjOut];
  int32_t out_type[kMaxProjOut];  // ColTypeCode
  int32_t n_out;
  int32_t pad;
  int64_t n;              // rows (capacity when n_dev is set)
  const int64_t* n_dev;   // deferred row count
  DevStatus* st;
};

__global__ void __launch_bounds__(256) project_kernel(const __grid_constant__ ProjectParams p) {
  int64_t n = p.n;
  if (p.n_dev != nullptr && *p.n_dev < n) n = *p.n_dev;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; row < n; row += stride) {
    for (int j = 0; j < p.n_out; ++j) {
      const int64_t v = operand_row(p.prog, p.cols, p.ops[j], row, p.st);
      if (p.out_type[j] == CT_I64 || p.out_type[j] == CT_F64)
        static_cast<int64_t*>(p.out[j])[row] = v;
      else
        static_cast<int32_t*>(p.out[j])[row] = static_cast<int32_t>(v);
    }
  }
}

// ------------------------------------------------------------------ top-k

constexpr int kSortThreads = 512;
constexpr int kSortChunk = 2048;  // row ids per block per round

struct SortKeyDev {
  DevCol col;
  int32_t desc;
  int32_t pad;
};

struct SelectKParams {
  SortKeyDev keys[kMaxSortKeys];
  int32_t n_keys;
  int32_t pad;
  const int32_t* in;     // row ids of this round (-1: none); nullptr: rows 0..n-1
  int64_t m;             // entries of `in` (or rows)
  const int64_t* n_dev;  // deferred row count (first round)
  int32_t* out;          // kk entries per block
  int32_t kk;            // entries each block keeps
};

// Order-preserving 64-bit prefix of key 0 of a row (descending keys
// inverted): equal prefixes fall back to the full comparison.
__device__ __forceinline__ uint64_t sort_prefix(const SortKeyDev& k, int32_t row) {
  uint64_t u;
  const DevCol& c = k.col;
  if (c.type == CT_UTF8) {
    const int32_t b = c.offsets[row], e = c.offsets[row + 1];
    const uint8_t* s = static_cast<const uint8_t*>(c.data);
    u = 0;
    for (int i = 0; i < 8; ++i) u = (u << 8) | (b + i < e ? s[b + i] : 0u);
  } else if (c.type == CT_F64) {
    const uint64_t bits = static_cast<uint64_t>(load_as_i64_bits(c, row));
    u = (bits >> 63) ? ~bits : bits | 0x8000000000000000ull;  // IEEE order (NaN with the sign bit clear sorts last)
  } else {
    u = static_cast<uint64_t>(load_int(c, row)) ^ 0x8000000000000000ull;
  }
  return k.desc ? ~u : u;
}

// Full three-way comparison of rows a and b on key i.
__device__ __forceinline__ int compare_key(const SortKeyDev& k, int32_t a, int32_t b) {
  const DevCol& c = k.col;
  int r = 0;
  if (c.type == CT_UTF8) {
    const int32_t ab = c.offsets[a], ae = c.offsets[a + 1], bb = c.offsets[b], be = c.offsets[b + 1];
    const uint8_t* s = static_cast<const uint8_t*>(c.data);
    const int32_t la = ae - ab, lb = be - bb;
    const int32_t n = la < lb ? la : lb;
    for (int32_t i = 0; i < n && r == 0; ++i) r = s[ab + i] < s[bb + i] ? -1 : s[ab + i] > s[bb + i] ? 1 : 0;
    if (r == 0) r = la < lb ? -1 : la > lb ? 1 : 0;
  } else if (c.type == CT_F64) {
    const uint64_t pa = sort_prefix(SortKeyDev{c, 0, 0}, a), pb = sort_prefix(SortKeyDev{c, 0, 0}, b);
    r = pa < pb ? -1 : pa > pb ? 1 : 0;
  } else {
    const int64_t va = load_int(c, a), vb = load_int(c, b);
    r = va < vb ? -1 : va > vb ? 1 : 0;
  }
  return k.desc ? -r : r;
}

// a before b: valid ids before -1, then the keys, then the row id.
__device__ __forceinline__ bool sort_before(const SelectKParams& p, int32_t a, uint64_t pa, int32_t b, uint64_t pb) {
  if (a < 0 || b < 0) return a >= 0 && b < 0;
  if (pa != pb) return pa < pb;
  for (int i = 0; i < p.n_keys; ++i) {
    // key 0's prefix is the whole key for fixed-width columns
    if (i == 0 && p.keys[0].col.type != CT_UTF8) continue;
    const int r = compare_key(p.keys[i], a, b);
    if (r != 0) return r < 0;
  }
  return a < b;
}

__global__ void __launch_bounds__(kSortThreads) select_k_kernel(const __grid_constant__ SelectKParams p) {
  __shared__ int32_t s_id[kSortChunk];
  __shared__ uint64_t s_pre[kSortChunk];
  int64_t m = p.m;
  if (p.in == nullptr && p.n_dev != nullptr && *p.n_dev < m) m = *p.n_dev;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kSortChunk;
  for (int i = threadIdx.x; i < kSortChunk; i += kSortThreads) {
    const int64_t j = base + i;
    int32_t id = -1;
    if (j < m) id = p.in != nullptr ? p.in[j] : static_cast<int32_t>(j);
    s_id[i] = id;
    s_pre[i] = id >= 0 ? sort_prefix(p.keys[0], id) : ~0ull;
  }
  __syncthreads();
  // bitonic sort of the chunk, ascending in sort_before order
  for (int size = 2; size <= kSortChunk; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < kSortChunk / 2; t += kSortThreads) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const int32_t a = s_id[lo], b = s_id[hi];
        const uint64_t pa = s_pre[lo], pb = s_pre[hi];
        const bool swap = up ? sort_before(p, b, pb, a, pa) : sort_before(p, a, pa, b, pb);
        if (swap) {
          s_id[lo] = b;
          s_id[hi] = a;
          s_pre[lo] = pb;
          s_pre[hi] = pa;
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < p.kk; i += kSortThreads) p.out[static_cast<int64_t>(blockIdx.x) * p.kk + i] = s_id[i];
}

int grid_rows(int64_t n) {
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = static_cast<int64_t>(num_sms()) * 8;
  if (blocks > cap) blocks = cap;
  return static_cast<int>(blocks < 1 ? 1 : blocks);
}

}  // namespace

namespace {

__global__ void substr_lengths_kernel(const int32_t* __restrict__ offs, int64_t n, int sub, int from, int len,
                                      int32_t* __restrict__ out_len) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t b = offs[r], e = offs[r + 1];
    if (sub) substring_range(&b, &e, from, len);
    out_len[r] = e - b;
  }
}

__global__ void substr_copy_kernel(const int32_t* __restrict__ offs, const uint8_t* __restrict__ bytes, int64_t n,
                                   int sub, int from, int len, const int32_t* __restrict__ out_offs,
                                   uint8_t* __restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    int32_t b = offs[r], e = offs[r + 1];
    if (sub) substring_range(&b, &e, from, len);
    const int32_t o = out_offs[r];
    for (int32_t k = 0; k < e - b; ++k) out[o + k] = bytes[b + k];
  }
}

}  // namespace

ColumnPtr substring_column(const Column& c, int64_t n, bool sub, int from, int len, cudaStream_t s) {
  if (c.type != DType::Utf8) fail(GFPDB_EINVAL, "substring of a column that is not utf8");
  auto offs = make_buffer((n + 1) * 4, s);
  int64_t total = 0;
  if (n > 0) {
    auto lens = make_buffer(n * 4, s);
    substr_lengths_kernel<<<grid_rows(n), 256, 0, s>>>(c.offsets, n, sub ? 1 : 0, from, len, lens->as<int32_t>());
    after_launch("substr_lengths_kernel");
    total = exclusive_scan_i32(lens->as<int32_t>(), offs->as<int32_t>(), n, s);
  } else {
    GF_CUDA(cudaMemsetAsync(offs->data(), 0, 4, s));
  }
  auto bytes = make_buffer(total > 0 ? total : 1, s);
  if (n > 0 && total > 0) {
    substr_copy_kernel<<<grid_rows(n), 256, 0, s>>>(c.offsets, static_cast<const uint8_t*>(c.data), n, sub ? 1 : 0,
                                                    from, len, offs->as<int32_t>(), bytes->as<uint8_t>());
    after_launch("substr_copy_kernel");
  }
  return make_utf8_column(n, offs, bytes);
}

TupleSetPtr project_columns(const ProjectSpec& spec, const TupleSet& in, cudaStream_t s) {
  const int n_out = static_cast<int>(spec.ops.size());
  if (n_out > kMaxProjOut) fail(GFPDB_EUNSUPPORTED, "more than 16 projected expressions in one operator");
  ProjectParams p;
  std::memset(&p, 0, sizeof(p));
  p.prog = spec.prog;
  bind_columns(spec.slots, in, p.cols, kMaxCols);
  const int64_t cap = in.num_rows();
  std::vector<Field> fields;
  std::vector<ColumnPtr> cols;
  for (int j = 0; j < n_out; ++j) {
    const DType t = spec.types[j];
    if (t == DType::Utf8) fail(GFPDB_EUNSUPPORTED, "utf8-valued projected expressions");
    auto buf = make_buffer(cap * dtype_width(t), s);
    p.ops[j] = spec.ops[j];
    p.out[j] = buf->data();
    p.out_type[j] = static_cast<int32_t>(t);
    fields.push_back(Field{spec.names[j], t});
    cols.push_back(make_fixed_column(t, cap, buf));
  }
  p.n_out = n_out;
  p.n = cap;
  p.n_dev = in.rows_dev();
  auto status = make_filled(sizeof(DevStatus), 0, s);
  p.st = status->as<DevStatus>();
  if (cap > 0 && n_out > 0) {
    ProfScope prof("project_kernel", s);
    project_kernel<<<grid_rows(cap), 256, 0, s>>>(p);
    after_launch("project_kernel");
    prof.stop(static_cast<double>(cap) * 8.0 * n_out);
  }
  if (deferred_mode())
    defer_check(status, status->as<DevStatus>(), "ProjectPOp expression");
  else
  {
    DevStatus h;
    GF_CUDA(cudaMemcpyAsync(&h, status->data(), sizeof(h), cudaMemcpyDeviceToHost, s));
    sync(s);
    raise_device_status(h, "ProjectPOp expression");
  }
  if (in.exact()) return TupleSet::make(std::move(fields), std::move(cols), cap);
  return TupleSet::make_deferred(std::move(fields), std::move(cols), cap, in.rows_owner(), in.rows_dev());
}

TupleSetPtr select_k(const TupleSetPtr& input, const std::vector<SortKeySpec>& keys, int64_t k, cudaStream_t s) {
  if (keys.empty() || keys.size() > static_cast<size_t>(kMaxSortKeys))
    fail(GFPDB_EUNSUPPORTED, "LimitSortPOp takes 1 to 4 sort keys");
  if (k < 0) fail(GFPDB_EINVAL, "LimitSortPOp limit must not be negative");
  if (k > kSortChunk / 2) fail(GFPDB_EUNSUPPORTED, "LimitSortPOp limit above 1024 rows");
  const TupleSetPtr in = resolved(input, s);  // the output size needs the row count
  const int64_t n = in->num_rows();
  if (n > INT32_MAX) fail(GFPDB_EUNSUPPORTED, "LimitSortPOp input above 2^31 rows");
  SelectKParams p;
  std::memset(&p, 0, sizeof(p));
  for (size_t i = 0; i < keys.size(); ++i) {
    const auto& c = in->column(keys[i].column);
    p.keys[i].col = DevCol{c->data, c->offsets, static_cast<int32_t>(c->type), 0};
    p.keys[i].desc = keys[i].descending ? 1 : 0;
  }
  p.n_keys = static_cast<int32_t>(keys.size());
  const int64_t kept = std::min<int64_t>(k, n);
  std::vector<GatherSpec> specs;
  if (kept > 0) {
    // rounds: each block keeps kk of its 2048 ids, until one block is left
    const int32_t kk = static_cast<int32_t>(std::max<int64_t>(kept, 1));
    int64_t m = n;
    BufferPtr cur;  // this round's ids (none in the first round: rows 0..n-1)
    for (;;) {
      const int64_t blocks = (m + kSortChunk - 1) / kSortChunk;
      auto next = make_buffer(blocks * kk * 4, s);
      p.in = cur ? cur->as<int32_t>() : nullptr;
      p.m = m;
      p.out = next->as<int32_t>();
      p.kk = kk;
      ProfScope prof("select_k_kernel", s);
      select_k_kernel<<<static_cast<int>(blocks), kSortThreads, 0, s>>>(p);
      after_launch("select_k_kernel");
      prof.stop(static_cast<double>(m) * 4.0);
      cur = next;
      m = blocks * kk;
      if (blocks == 1) break;
    }
    for (int i = 0; i < in->num_columns(); ++i) specs.push_back(GatherSpec{in->column(i).get(), cur->as<int32_t>()});
    auto cols = gather_columns(specs, kept, s);
    return TupleSet::make(in->fields(), std::move(cols), kept);
  }
  return TupleSet::make_empty(in->fields(), s);
}

}  // namespace gfpdb
