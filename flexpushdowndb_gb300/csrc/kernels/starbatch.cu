// Batched star queries: many query variants over one partitioned fact table,
// one launch per stage for all of them.
//
// The single-query plan runs each operator of the reference's star plan
// (dimension FilterPOps, forward and backward bloom filters, four
// HashJoinArrowPOps and a GroupPOp, SmallToLargePredTransOrder.cpp:38-214)
// once per query. Here Q queries that differ only in their dimension filter
// ranges share every scan:
//   stage 1 (one launch, all dimensions): each dimension row gets the bitmask
//     of the queries whose range selects it, and rows selected by any query
//     go into one shared open-addressing join table per dimension;
//   stage 2 (one persistent launch over every tile of every partition): a
//     fact row probes each dimension's table once for all queries, ANDs the
//     rows' query masks (most selective dimension first, stopping at zero),
//     and for each query left adds its measures into that query's group
//     table (int64 two's-complement sums, exact);
//   stage 3 (one launch): every query's groups are compacted into one output
//     with a query_id column.
// The per-dimension masks are exact, so the single-query bloom filters (a
// pre-filter whose false positives the joins remove anyway) have nothing left
// to do and are not built; each query's result is bit-identical to its
// single-query plan. Dimension keys must be unique (star schema primary
// keys); a repeated key is reported as an error.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "launch.h"

namespace gfpdb {

namespace sb {

constexpr int kSBThreads = 256;

struct SBDimDev {
  DevCol key;
  DevCol filter;
  DevCol group[2];       // group columns carried by this dimension (type -1: none)
  int64_t rows;
  int64_t row_base;      // offset of this dimension in the flattened stage-1 index
  uint64_t* slots;       // (tag << 32 | row), all-ones = empty
  uint64_t mask;         // capacity - 1
  uint64_t* qmask;       // per dimension row
  int32_t key32;
  int32_t n_group;
};

struct SBDimsParams {
  SBDimDev dims[kSBMaxDims];
  int32_t n_dims;
  int32_t n_queries;
  int64_t total_rows;
  const int64_t* ranges;  // [q][d][2] (lo, hi)
  DevStatus* st;
};

__global__ void __launch_bounds__(kSBThreads) sb_dims_kernel(const __grid_constant__ SBDimsParams p) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < p.total_rows; i += stride) {
    int d = 0;
    while (d + 1 < p.n_dims && i >= p.dims[d + 1].row_base) ++d;
    const SBDimDev& D = p.dims[d];
    const int64_t r = i - D.row_base;
    const int64_t v = load_int(D.filter, r);
    uint64_t m = 0;
    for (int q = 0; q < p.n_queries; ++q) {
      const int64_t* rg = p.ranges + (static_cast<int64_t>(q) * kSBMaxDims + d) * 2;
      if (rg[0] <= v && v <= rg[1]) m |= 1ull << q;
    }
    D.qmask[r] = m;
    if (m == 0) continue;
    const int64_t k = load_int(D.key, r);
    const uint64_t h = hash_key(k);
    const uint32_t tag = D.key32 ? static_cast<uint32_t>(k) : static_cast<uint32_t>(h >> 32);
    const uint64_t packed = (static_cast<uint64_t>(tag) << 32) | static_cast<uint32_t>(r);
    uint64_t slot = h & D.mask;
    bool placed = false;
    for (uint64_t probe = 0; probe <= D.mask; ++probe) {
      const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long*>(D.slots + slot),
                                               static_cast<unsigned long long>(kEmptySlot),
                                               static_cast<unsigned long long>(packed));
      if (old == kEmptySlot) {
        placed = true;
        break;
      }
      if (static_cast<uint32_t>(old >> 32) == tag && (D.key32 || load_int(D.key, static_cast<uint32_t>(old)) == k)) {
        raise_status(p.st, GFPDB_EINVAL, 100 + d);  // repeated dimension key
        placed = true;
        break;
      }
      slot = (slot + 1) & D.mask;
    }
    if (!placed) raise_status(p.st, GFPDB_ENOMEM, 110 + d);
  }
}

struct SBFactDims {
  int32_t fk_col[kSBMaxDims];  // fact column slot of each dimension's foreign key
  int32_t order[kSBMaxDims];   // probe order
  int32_t group_dim[2];        // dimension carrying group column g (or -1)
  int32_t group_idx[2];        // which of that dimension's group columns
  int32_t n_group;
  int32_t pad;
};

struct SBAgg {
  int32_t fn;     // AGG_SUM / AGG_COUNT_STAR
  int32_t a, b;   // fact column slots (b < 0: single column)
  int32_t pad;
};

struct SBFactParams {
  SBDimDev dims[kSBMaxDims];
  SBFactDims fd;
  SBAgg aggs[kMaxAggs];
  int32_t n_dims;
  int32_t n_aggs;
  int32_t n_queries;
  int32_t n_parts;
  int32_t n_cols;       // fact columns per partition
  int32_t items;        // rows per thread per tile
  uint64_t qvalid;      // bitmask of the batch's queries
  const DevCol* part_cols;   // [part][n_cols]
  const int64_t* tile_base;  // [n_parts + 1] first tile of each partition
  const int64_t* part_rows;  // [n_parts]
  int64_t n_tiles;
  uint32_t* ticket;
  uint64_t* gkeys;           // [q][gcap + 1]
  unsigned long long* gaccs; // [q][gcap + 1][n_aggs]
  uint64_t gmask;            // gcap - 1
  int64_t* special;          // [q] the all-ones key has a group
  int64_t* groups;           // [q] groups claimed
  DevStatus* st;
};

__device__ __forceinline__ int64_t sb_lookup(const SBDimDev& D, int64_t k) {
  const uint64_t h = hash_key(k);
  const uint32_t tag = D.key32 ? static_cast<uint32_t>(k) : static_cast<uint32_t>(h >> 32);
  uint64_t slot = h & D.mask;
  for (uint64_t probe = 0; probe <= D.mask; ++probe) {
    const uint64_t s = __ldg(reinterpret_cast<const unsigned long long*>(D.slots + slot));
    if (s == kEmptySlot) return -1;
    if (static_cast<uint32_t>(s >> 32) == tag) {
      const int64_t r = static_cast<uint32_t>(s);
      if (D.key32 || load_int(D.key, r) == k) return r;
    }
    slot = (slot + 1) & D.mask;
  }
  return -1;
}

__device__ __forceinline__ uint64_t sb_group_slot(const SBFactParams& p, int q, uint64_t key) {
  uint64_t* keys = p.gkeys + static_cast<uint64_t>(q) * (p.gmask + 2);
  if (key == kEmptySlot) {
    if (atomicExch(reinterpret_cast<unsigned long long*>(&p.special[q]), 1ull) == 0ull)
      atomicAdd(reinterpret_cast<unsigned long long*>(&p.groups[q]), 1ull);
    return p.gmask + 1;
  }
  uint64_t slot = hash_key(static_cast<int64_t>(key)) & p.gmask;
  for (uint64_t i = 0; i <= p.gmask; ++i) {
    uint64_t s = *reinterpret_cast<volatile uint64_t*>(keys + slot);
    if (s == kEmptySlot) {
      s = atomicCAS(reinterpret_cast<unsigned long long*>(keys + slot), static_cast<unsigned long long>(kEmptySlot),
                    static_cast<unsigned long long>(key));
      if (s == kEmptySlot) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&p.groups[q]), 1ull);
        return slot;
      }
    }
    if (s == key) return slot;
    slot = (slot + 1) & p.gmask;
  }
  raise_status(p.st, GFPDB_ENOMEM, 120);
  return UINT64_MAX;
}

__global__ void __launch_bounds__(kSBThreads) sb_fact_kernel(const __grid_constant__ SBFactParams p) {
  __shared__ int64_t s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = static_cast<int64_t>(atomicAdd(p.ticket, 1u));
    __syncthreads();
    const int64_t tile = s_tile;
    __syncthreads();
    if (tile >= p.n_tiles) break;
    int part = 0;
    {
      int lo = 0, hi = p.n_parts - 1;  // last partition whose first tile <= tile
      while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (p.tile_base[mid] <= tile) lo = mid;
        else hi = mid - 1;
      }
      part = lo;
    }
    const DevCol* cols = p.part_cols + static_cast<int64_t>(part) * p.n_cols;
    const int64_t rows = p.part_rows[part];
    const int64_t row0 = (tile - p.tile_base[part]) * static_cast<int64_t>(kSBThreads) * p.items;
    for (int it = 0; it < p.items; ++it) {
      // consecutive threads read consecutive rows: coalesced FK loads
      const int64_t row = row0 + static_cast<int64_t>(it) * kSBThreads + threadIdx.x;
      if (row >= rows) break;
      uint64_t m = p.qvalid;
      int64_t drow[kSBMaxDims];
      for (int j = 0; j < p.n_dims && m != 0; ++j) {
        const int d = p.fd.order[j];
        const int64_t r = sb_lookup(p.dims[d], load_int(cols[p.fd.fk_col[d]], row));
        drow[d] = r;
        m &= r >= 0 ? __ldg(reinterpret_cast<const unsigned long long*>(p.dims[d].qmask + r)) : 0ull;
      }
      if (m == 0) continue;
      uint64_t key = 0;
      if (p.fd.n_group == 1) {
        const SBDimDev& D = p.dims[p.fd.group_dim[0]];
        key = static_cast<uint32_t>(load_int(D.group[p.fd.group_idx[0]], drow[p.fd.group_dim[0]]));
      } else if (p.fd.n_group == 2) {
        const SBDimDev& A = p.dims[p.fd.group_dim[0]];
        const SBDimDev& B = p.dims[p.fd.group_dim[1]];
        const uint32_t a = static_cast<uint32_t>(load_int(A.group[p.fd.group_idx[0]], drow[p.fd.group_dim[0]]));
        const uint32_t b = static_cast<uint32_t>(load_int(B.group[p.fd.group_idx[1]], drow[p.fd.group_dim[1]]));
        key = (static_cast<uint64_t>(a) << 32) | b;
      }
      unsigned long long vals[kMaxAggs];
      for (int a = 0; a < p.n_aggs; ++a) {
        const SBAgg& g = p.aggs[a];
        if (g.fn == AGG_COUNT_STAR) {
          vals[a] = 1ull;
        } else {
          uint64_t v = static_cast<uint64_t>(load_int(cols[g.a], row));
          if (g.b >= 0) v *= static_cast<uint64_t>(load_int(cols[g.b], row));  // int64 wrap
          vals[a] = v;
        }
      }
      while (m != 0) {
        const int q = __ffsll(static_cast<long long>(m)) - 1;
        m &= m - 1;
        const uint64_t slot = sb_group_slot(p, q, key);
        if (slot == UINT64_MAX) continue;
        unsigned long long* acc =
            p.gaccs + (static_cast<uint64_t>(q) * (p.gmask + 2) + slot) * static_cast<uint64_t>(p.n_aggs);
        for (int a = 0; a < p.n_aggs; ++a) atomicAdd(acc + a, vals[a]);
      }
    }
  }
}

struct SBFinalParams {
  const uint64_t* gkeys;
  const unsigned long long* gaccs;
  const int64_t* special;
  uint64_t slots_per_q;  // gcap + 1
  int32_t n_queries;
  int32_t n_aggs;
  int32_t n_group;
  int32_t group_type[2];
  int32_t* out_q;
  void* out_g[2];
  long long* out_a[kMaxAggs];
  unsigned long long* counter;
};

__global__ void __launch_bounds__(256) sb_final_kernel(const __grid_constant__ SBFinalParams p) {
  const int lane = threadIdx.x & 31;
  const uint64_t total = p.slots_per_q * static_cast<uint64_t>(p.n_queries);
  const uint64_t w0 = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t base = w0 * 32; base < total; base += nw * 32) {
    const uint64_t i = base + lane;
    bool live = false;
    uint64_t key = 0;
    int q = 0;
    if (i < total) {
      q = static_cast<int>(i / p.slots_per_q);
      const uint64_t s = i % p.slots_per_q;
      if (s + 1 < p.slots_per_q) {
        key = p.gkeys[i];
        live = key != kEmptySlot;
      } else {
        key = kEmptySlot;
        live = p.special[q] != 0;
      }
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, live);
    if (bal == 0) continue;
    unsigned long long at = 0;
    const int leader = __ffs(bal) - 1;
    if (lane == leader) at = atomicAdd(p.counter, static_cast<unsigned long long>(__popc(bal)));
    at = __shfl_sync(0xffffffffu, at, leader);
    if (!live) continue;
    const int64_t pos = static_cast<int64_t>(at) + __popc(bal & ((1u << lane) - 1u));
    p.out_q[pos] = q;
    if (p.n_group == 1) {
      const int32_t v = static_cast<int32_t>(static_cast<uint32_t>(key));
      static_cast<int32_t*>(p.out_g[0])[pos] = v;
    } else if (p.n_group == 2) {
      static_cast<int32_t*>(p.out_g[0])[pos] = static_cast<int32_t>(static_cast<uint32_t>(key >> 32));
      static_cast<int32_t*>(p.out_g[1])[pos] = static_cast<int32_t>(static_cast<uint32_t>(key));
    }
    for (int a = 0; a < p.n_aggs; ++a) p.out_a[a][pos] = static_cast<long long>(p.gaccs[i * p.n_aggs + a]);
  }
}

uint64_t pow2_at_least(uint64_t x) {
  uint64_t c = 64;
  while (c < x) c <<= 1;
  return c;
}

}  // namespace sb

// ----------------------------------------------------------------- host side

using namespace sb;

struct StarBatchState {
  StarBatchSpec spec;
  std::vector<TupleSetPtr> parts, dim_tables;
  std::vector<std::string> fact_cols;
  SBDimsParams dims_params;
  SBFactParams fact_params;
  BufferPtr tables_buf, masks_buf, gkeys_buf, gaccs_buf, misc_buf, meta_buf, out_q;
  BufferPtr out_g[2], out_a[kMaxAggs];
  std::vector<char> host_meta;
  DType group_types[2] = {DType::Int32, DType::Int32};
  uint64_t gcap = 0;
  int64_t out_cap = 0, n_tiles = 0, fact_rows = 0;
  unsigned long long* counter = nullptr;

  void prepare(cudaStream_t s);
  void run(cudaStream_t s);
  TupleSetPtr result_view() const;
  const DevStatus* status() const;
};

StarBatch::StarBatch() : st_(new StarBatchState()) {}
StarBatch::~StarBatch() = default;
StarBatchSpec& StarBatch::spec() { return st_->spec; }
std::vector<TupleSetPtr>& StarBatch::parts() { return st_->parts; }
std::vector<TupleSetPtr>& StarBatch::dim_tables() { return st_->dim_tables; }
void StarBatch::prepare(cudaStream_t s) { st_->prepare(s); }
void StarBatch::run(cudaStream_t s) { st_->run(s); }
TupleSetPtr StarBatch::result_view() const { return st_->result_view(); }
const DevStatus* StarBatch::status() const { return st_->status(); }
int64_t StarBatch::fact_rows() const { return st_->fact_rows; }

void StarBatchState::prepare(cudaStream_t s) {
  if (spec.dims.empty() || spec.dims.size() > static_cast<size_t>(kSBMaxDims))
    fail(GFPDB_EUNSUPPORTED, "a batched star query needs 1 to 8 dimensions");
  if (spec.queries.empty() || spec.queries.size() > static_cast<size_t>(kSBMaxQueries))
    fail(GFPDB_EUNSUPPORTED, "a batch holds 1 to 64 queries");
  if (spec.group.size() > 2) fail(GFPDB_EUNSUPPORTED, "at most two group columns in a batched star query");
  if (spec.aggs.empty() || spec.aggs.size() > static_cast<size_t>(kMaxAggs))
    fail(GFPDB_EUNSUPPORTED, "1 to 8 aggregates in a batched star query");
  if (parts.empty() || parts.size() > static_cast<size_t>(kSBMaxParts))
    fail(GFPDB_EUNSUPPORTED, "a batch scans 1 to 256 fact partitions");
  const int nd = static_cast<int>(spec.dims.size());
  const int nq = static_cast<int>(spec.queries.size());
  // fact columns: every foreign key, then every measure column
  fact_cols.clear();
  auto slot_of = [&](const std::string& name) {
    for (size_t i = 0; i < fact_cols.size(); ++i)
      if (fact_cols[i] == name) return static_cast<int>(i);
    fact_cols.push_back(name);
    return static_cast<int>(fact_cols.size()) - 1;
  };
  std::vector<int> fk_slot(nd), agg_a(spec.aggs.size(), -1), agg_b(spec.aggs.size(), -1);
  for (int d = 0; d < nd; ++d) fk_slot[d] = slot_of(spec.dims[d].fact_key);
  for (size_t a = 0; a < spec.aggs.size(); ++a) {
    if (spec.aggs[a].fn == AGG_COUNT_STAR) continue;
    if (spec.aggs[a].columns.empty() || spec.aggs[a].columns.size() > 2)
      fail(GFPDB_EUNSUPPORTED, "a batched SUM takes one column or the product of two");
    agg_a[a] = slot_of(spec.aggs[a].columns[0]);
    if (spec.aggs[a].columns.size() == 2) agg_b[a] = slot_of(spec.aggs[a].columns[1]);
  }
  const int nc = static_cast<int>(fact_cols.size());
  // partitions: column descriptors and tile ranges
  const int items = spec.items_per_thread;
  if (items < 1 || items > 64) fail(GFPDB_EINVAL, "itemsPerThread must be in [1, 64]");
  const int64_t tile_rows = static_cast<int64_t>(kSBThreads) * items;
  std::vector<DevCol> hcols(parts.size() * nc);
  std::vector<int64_t> hbase(parts.size() + 1), hrows(parts.size());
  int64_t tiles = 0;
  fact_rows = 0;
  for (size_t pi = 0; pi < parts.size(); ++pi) {
    const TupleSet& t = *parts[pi];
    if (!t.exact()) fail(GFPDB_EINVAL, "batched star partitions must have exact row counts");
    for (int c = 0; c < nc; ++c) {
      const auto& col = t.column(fact_cols[c]);
      if (col->type == DType::Utf8 || col->type == DType::Float64)
        fail(GFPDB_EUNSUPPORTED, "batched star fact columns must be integer columns");
      hcols[pi * nc + c] = DevCol{col->data, nullptr, static_cast<int32_t>(col->type), 0};
    }
    hbase[pi] = tiles;
    hrows[pi] = t.num_rows();
    tiles += (t.num_rows() + tile_rows - 1) / tile_rows;
    fact_rows += t.num_rows();
  }
  hbase[parts.size()] = tiles;
  n_tiles = tiles;
  // dimensions
  std::memset(&dims_params, 0, sizeof(dims_params));
  int64_t base = 0;
  for (int d = 0; d < nd; ++d) {
    const auto& ds = spec.dims[d];
    const TupleSet& t = *dim_tables[d];
    if (!t.exact()) fail(GFPDB_EINVAL, "batched star dimensions must have exact row counts");
    SBDimDev& D = dims_params.dims[d];
    const auto& key = t.column(ds.key);
    const auto& filt = t.column(ds.filter);
    if (key->type == DType::Utf8 || key->type == DType::Float64 || filt->type == DType::Utf8 ||
        filt->type == DType::Float64)
      fail(GFPDB_EUNSUPPORTED, "batched star keys and filter columns must be integer columns");
    D.key = DevCol{key->data, nullptr, static_cast<int32_t>(key->type), 0};
    D.filter = DevCol{filt->data, nullptr, static_cast<int32_t>(filt->type), 0};
    D.group[0].type = D.group[1].type = -1;
    D.rows = t.num_rows();
    D.row_base = base;
    base += t.num_rows();
    const uint64_t cap = pow2_at_least(static_cast<uint64_t>(static_cast<double>(t.num_rows()) / spec.load_factor) + 1);
    D.mask = cap - 1;
    D.key32 = key->type != DType::Int64;
  }
  dims_params.n_dims = nd;
  dims_params.n_queries = nq;
  dims_params.total_rows = base;
  // group columns
  std::memset(&fact_params, 0, sizeof(fact_params));
  fact_params.fd.n_group = static_cast<int32_t>(spec.group.size());
  for (size_t g = 0; g < spec.group.size(); ++g) {
    const int d = spec.group[g].dim;
    if (d < 0 || d >= nd) fail(GFPDB_EINVAL, "group column names an unknown dimension");
    SBDimDev& D = dims_params.dims[d];
    const auto& c = dim_tables[d]->column(spec.group[g].column);
    if (c->type == DType::Utf8 || c->type == DType::Float64 || c->type == DType::Int64)
      fail(GFPDB_EUNSUPPORTED, "batched star group columns must be int32 or date32");
    D.group[D.n_group] = DevCol{c->data, nullptr, static_cast<int32_t>(c->type), 0};
    fact_params.fd.group_dim[g] = d;
    fact_params.fd.group_idx[g] = D.n_group;
    group_types[g] = c->type;
    ++D.n_group;
  }
  for (int d = 0; d < nd; ++d) {
    fact_params.fd.fk_col[d] = fk_slot[d];
    fact_params.fd.order[d] = d < static_cast<int>(spec.probe_order.size()) ? spec.probe_order[d] : d;
  }
  for (size_t a = 0; a < spec.aggs.size(); ++a) {
    fact_params.aggs[a].fn = spec.aggs[a].fn == AGG_COUNT_STAR ? AGG_COUNT_STAR : AGG_SUM;
    fact_params.aggs[a].a = agg_a[a];
    fact_params.aggs[a].b = agg_b[a];
  }
  // device buffers (allocated once; a run only clears and fills them)
  int64_t table_words = 0, mask_words = 0;
  for (int d = 0; d < nd; ++d) {
    table_words += static_cast<int64_t>(dims_params.dims[d].mask + 1);
    mask_words += dims_params.dims[d].rows;
  }
  gcap = pow2_at_least(static_cast<uint64_t>(2 * std::max<int64_t>(spec.groups_hint, 16)));
  const int na = static_cast<int>(spec.aggs.size());
  const int64_t gslots = static_cast<int64_t>(nq) * static_cast<int64_t>(gcap + 1);
  tables_buf = make_buffer(table_words * 8, s);
  masks_buf = make_buffer(std::max<int64_t>(mask_words, 1) * 8, s);
  gkeys_buf = make_buffer(gslots * 8, s);
  gaccs_buf = make_buffer(gslots * 8 * na, s);
  misc_buf = make_buffer(sizeof(DevStatus) + 64 + 2 * 8 * kSBMaxQueries + 64, s);
  meta_buf = make_buffer(static_cast<int64_t>(hcols.size() * sizeof(DevCol) + hbase.size() * 8 + hrows.size() * 8 +
                                              kSBMaxQueries * kSBMaxDims * 16),
                         s);
  out_cap = gslots;
  out_q = make_buffer(out_cap * 4, s);
  for (size_t g = 0; g < spec.group.size(); ++g) out_g[g] = make_buffer(out_cap * 4, s);
  for (int a = 0; a < na; ++a) out_a[a] = make_buffer(out_cap * 8, s);
  // wire pointers
  int64_t toff = 0, moff = 0;
  for (int d = 0; d < nd; ++d) {
    SBDimDev& D = dims_params.dims[d];
    D.slots = tables_buf->as<uint64_t>() + toff;
    D.qmask = masks_buf->as<uint64_t>() + moff;
    toff += static_cast<int64_t>(D.mask + 1);
    moff += D.rows;
  }
  char* misc = misc_buf->as<char>();
  DevStatus* st = reinterpret_cast<DevStatus*>(misc);
  dims_params.st = st;
  char* meta = meta_buf->as<char>();
  DevCol* dcols = reinterpret_cast<DevCol*>(meta);
  int64_t* dbase = reinterpret_cast<int64_t*>(meta + hcols.size() * sizeof(DevCol));
  int64_t* drows = dbase + hbase.size();
  int64_t* dranges = drows + hrows.size();
  dims_params.ranges = dranges;
  // Metadata goes up once, from host memory that this object keeps (so a
  // captured graph never needs it again).
  host_meta.assign(meta_buf->size(), 0);
  std::memcpy(host_meta.data(), hcols.data(), hcols.size() * sizeof(DevCol));
  std::memcpy(host_meta.data() + hcols.size() * sizeof(DevCol), hbase.data(), hbase.size() * 8);
  std::memcpy(host_meta.data() + hcols.size() * sizeof(DevCol) + hbase.size() * 8, hrows.data(), hrows.size() * 8);
  int64_t* hr = reinterpret_cast<int64_t*>(host_meta.data() + hcols.size() * sizeof(DevCol) + hbase.size() * 8 +
                                           hrows.size() * 8);
  for (int q = 0; q < nq; ++q)
    for (int d = 0; d < nd; ++d) {
      hr[(q * kSBMaxDims + d) * 2] = spec.queries[q][d].first;
      hr[(q * kSBMaxDims + d) * 2 + 1] = spec.queries[q][d].second;
    }
  GF_CUDA(cudaMemcpyAsync(meta, host_meta.data(), host_meta.size(), cudaMemcpyHostToDevice, s));
  sync(s);
  fact_params.n_dims = nd;
  fact_params.n_aggs = na;
  fact_params.n_queries = nq;
  fact_params.n_parts = static_cast<int32_t>(parts.size());
  fact_params.n_cols = nc;
  fact_params.items = items;
  fact_params.qvalid = nq == 64 ? ~0ull : ((1ull << nq) - 1);
  fact_params.part_cols = dcols;
  fact_params.tile_base = dbase;
  fact_params.part_rows = drows;
  fact_params.n_tiles = n_tiles;
  fact_params.ticket = reinterpret_cast<uint32_t*>(misc + sizeof(DevStatus));
  fact_params.gkeys = gkeys_buf->as<uint64_t>();
  fact_params.gaccs = gaccs_buf->as<unsigned long long>();
  fact_params.gmask = gcap - 1;
  fact_params.special = reinterpret_cast<int64_t*>(misc + sizeof(DevStatus) + 64);
  fact_params.groups = fact_params.special + kSBMaxQueries;
  fact_params.st = st;
  for (int d = 0; d < nd; ++d) fact_params.dims[d] = dims_params.dims[d];
  counter = reinterpret_cast<unsigned long long*>(misc + sizeof(DevStatus) + 64 + 2 * 8 * kSBMaxQueries);
}

void StarBatchState::run(cudaStream_t s) {
  // clear: join tables to empty, group keys to empty, accumulators / status / counters to zero
  GF_CUDA(cudaMemsetAsync(tables_buf->data(), 0xFF, tables_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(gkeys_buf->data(), 0xFF, gkeys_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(gaccs_buf->data(), 0, gaccs_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(misc_buf->data(), 0, misc_buf->size(), s));
  const int sms = num_sms();
  {
    int64_t blocks = (dims_params.total_rows + kSBThreads - 1) / kSBThreads;
    if (blocks > sms * 8) blocks = sms * 8;
    if (blocks < 1) blocks = 1;
    ProfScope prof("sb_dims_kernel", s);
    sb_dims_kernel<<<static_cast<int>(blocks), kSBThreads, 0, s>>>(dims_params);
    after_launch("sb_dims_kernel");
    prof.stop(static_cast<double>(dims_params.total_rows) * 12.0);
  }
  if (n_tiles > 0) {
    int64_t grid = static_cast<int64_t>(sms) * spec.blocks_per_sm;
    if (grid > n_tiles) grid = n_tiles;
    ProfScope prof("sb_fact_kernel", s);
    sb_fact_kernel<<<static_cast<int>(grid), kSBThreads, 0, s>>>(fact_params);
    after_launch("sb_fact_kernel");
    // algorithmic bytes: every foreign key of every fact row read once
    prof.stop(static_cast<double>(fact_rows) * 4.0 * static_cast<double>(spec.dims.size()));
  }
  {
    SBFinalParams fp;
    std::memset(&fp, 0, sizeof(fp));
    fp.gkeys = gkeys_buf->as<uint64_t>();
    fp.gaccs = gaccs_buf->as<unsigned long long>();
    fp.special = fact_params.special;
    fp.slots_per_q = gcap + 1;
    fp.n_queries = static_cast<int32_t>(spec.queries.size());
    fp.n_aggs = static_cast<int32_t>(spec.aggs.size());
    fp.n_group = static_cast<int32_t>(spec.group.size());
    fp.out_q = out_q->as<int32_t>();
    for (size_t g = 0; g < spec.group.size(); ++g) fp.out_g[g] = out_g[g]->data();
    for (size_t a = 0; a < spec.aggs.size(); ++a) fp.out_a[a] = out_a[a]->as<long long>();
    fp.counter = counter;
    const uint64_t total = fp.slots_per_q * static_cast<uint64_t>(fp.n_queries);
    int64_t blocks = static_cast<int64_t>((total + 255) / 256);
    if (blocks > sms * 8) blocks = sms * 8;
    sb_final_kernel<<<static_cast<int>(blocks), 256, 0, s>>>(fp);
    after_launch("sb_final_kernel");
  }
}

TupleSetPtr StarBatchState::result_view() const {
  std::vector<Field> fields{Field{"query_id", DType::Int32}};
  std::vector<ColumnPtr> cols{make_fixed_column(DType::Int32, out_cap, out_q)};
  for (size_t g = 0; g < spec.group.size(); ++g) {
    fields.push_back(Field{spec.group[g].column, group_types[g]});
    cols.push_back(make_fixed_column(group_types[g], out_cap, out_g[g]));
  }
  for (size_t a = 0; a < spec.aggs.size(); ++a) {
    fields.push_back(Field{spec.aggs[a].name, DType::Int64});
    cols.push_back(make_fixed_column(DType::Int64, out_cap, out_a[a]));
  }
  return TupleSet::make_deferred(std::move(fields), std::move(cols), out_cap, misc_buf,
                                 reinterpret_cast<const int64_t*>(counter));
}

const DevStatus* StarBatchState::status() const { return misc_buf->as<DevStatus>(); }

}  // namespace gfpdb
