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
#include <mutex>

#include "common.cuh"
#include "launch.h"

namespace gfpdb {

namespace sb {

constexpr int kSBThreads = 256;

// A dimension is looked up in one of two ways, chosen on the device each run
// from the key range of its rows: when max - min + 1 is at most the table
// capacity (dense surrogate keys), the query mask and row of key k sit at
// k - min in two direct arrays; otherwise in the open-addressing table.
// Either way a fact row finds exactly the dimension rows whose key equals
// its foreign key.
struct SBDimDev {
  DevCol key;
  DevCol filter;
  DevCol group[2];       // group columns carried by this dimension (type -1: none)
  int64_t rows;
  int64_t row_base;      // offset of this dimension in the flattened stage-1 index
  uint64_t* slots;       // (tag << 32 | row), all-ones = empty
  uint64_t mask;         // capacity - 1
  uint64_t* qmask;       // per dimension row
  uint64_t* dq;          // direct: query mask per key - min (0 = no row)
  uint32_t* drow;        // direct: row per key - min (all-ones = no row)
  int32_t* dg[2];        // direct: group column values per key - min
  uint8_t* dclass;       // direct: segment class per key - min (kSBNoRow: no selected row)
  unsigned long long* kmin_u;  // key range, order-preserving unsigned (key ^ sign bit)
  unsigned long long* kmax_u;
  int32_t key32;
  int32_t n_group;
  int32_t smem_off;      // byte offset of this dimension's staged masks and group values (-1: not staged)
  int32_t smem_cap;      // keys staged when the key range fits (a multiple of 8)
};

// The queries' ranges on one dimension's filter column, as segments: the
// distinct range ends (every lo and hi + 1) cut the values into at most
// 2 * kSBMaxQueries + 1 segments, and within a segment every value is
// selected by the same queries. A row's query mask is then cmask[its
// segment], so a dimension row is described by one byte (its segment class)
// instead of a 4- or 8-byte mask: staged in shared memory, a dimension takes
// a quarter to an eighth of the room.
constexpr int kSBMaxBounds = 2 * kSBMaxQueries;
constexpr int kSBNoRow = 255;  // class of a key with no selected dimension row (mask 0)

struct SBSegments {
  int64_t n_bounds;
  int64_t bounds[kSBMaxBounds];   // ascending, distinct
  unsigned long long cmask[256];  // segment (number of bounds <= value) -> query mask; kSBNoRow: 0
};

// Segment of value v: the number of bounds <= v (binary search).
__device__ __forceinline__ int sb_segment(const SBSegments& S, int64_t v) {
  int lo = 0, hi = static_cast<int>(S.n_bounds);
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (S.bounds[mid] <= v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

struct SBDimsParams {
  SBDimDev dims[kSBMaxDims];
  int32_t n_dims;
  int32_t n_queries;
  int64_t total_rows;
  const SBSegments* segs;  // [dimension]
  DevStatus* st;
};

constexpr unsigned long long kSignBit = 0x8000000000000000ull;

struct SBDirect {
  int64_t kmin;
  uint64_t range;  // 0: look up in the hash table
};

__device__ __forceinline__ SBDirect sb_direct(const SBDimDev& D) {
  const unsigned long long lo = *reinterpret_cast<volatile unsigned long long*>(D.kmin_u);
  const unsigned long long hi = *reinterpret_cast<volatile unsigned long long*>(D.kmax_u);
  if (D.rows == 0 || lo > hi) return SBDirect{0, 0};
  const uint64_t range = static_cast<uint64_t>(hi - lo) + 1;  // difference of order-preserving codes
  if (range == 0 || range > D.mask + 1) return SBDirect{0, 0};
  return SBDirect{static_cast<int64_t>(lo ^ kSignBit), range};
}

// Key range of every dimension: blockIdx.y is the dimension.
__global__ void __launch_bounds__(kSBThreads) sb_range_kernel(const __grid_constant__ SBDimsParams p) {
  const SBDimDev& D = p.dims[blockIdx.y];
  unsigned long long lo = ~0ull, hi = 0ull;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < D.rows; r += stride) {
    const unsigned long long u = static_cast<unsigned long long>(load_int(D.key, r)) ^ kSignBit;
    lo = u < lo ? u : lo;
    hi = u > hi ? u : hi;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o);
    const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi, o);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if ((threadIdx.x & 31) == 0 && lo <= hi) {
    atomicMin(D.kmin_u, lo);
    atomicMax(D.kmax_u, hi);
  }
}

__global__ void __launch_bounds__(kSBThreads) sb_dims_kernel(const __grid_constant__ SBDimsParams p) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < p.total_rows; i += stride) {
    int d = 0;
    while (d + 1 < p.n_dims && i >= p.dims[d + 1].row_base) ++d;
    const SBDimDev& D = p.dims[d];
    const int64_t r = i - D.row_base;
    const int64_t v = load_int(D.filter, r);
    const int seg = sb_segment(p.segs[d], v);
    const uint64_t m = p.segs[d].cmask[seg];
    D.qmask[r] = m;
    if (m == 0) continue;
    const int64_t k = load_int(D.key, r);
    const SBDirect dr = sb_direct(D);
    if (dr.range != 0) {
      const uint64_t idx = static_cast<uint64_t>(k) - static_cast<uint64_t>(dr.kmin);  // < range by construction
      if (atomicCAS(D.drow + idx, 0xFFFFFFFFu, static_cast<uint32_t>(r)) != 0xFFFFFFFFu) {
        raise_status(p.st, GFPDB_EINVAL, 100 + d);  // repeated dimension key
      } else {
        D.dq[idx] = m;
        D.dclass[idx] = static_cast<uint8_t>(seg);
        for (int c = 0; c < D.n_group; ++c) D.dg[c][idx] = static_cast<int32_t>(load_int(D.group[c], r));
      }
      continue;
    }
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

constexpr int kSBConsumerWarps = 8;
constexpr int kSBFactThreads = (kSBConsumerWarps + 1) * 32;  // consumer warps + one producer warp
constexpr int kSBMaxStages = 8;
constexpr int kSBMaxAggsFact = 4;  // aggregates of a batched star query
constexpr int kSBBarBytes = 256;  // 2 * kSBMaxStages mbarriers, then the staging barrier

struct SBFactParams {
  SBDimDev dims[kSBMaxDims];
  SBFactDims fd;
  SBAgg aggs[kMaxAggs];
  int32_t n_dims;
  int32_t n_aggs;
  int32_t n_queries;
  int32_t n_parts;
  int32_t n_cols;       // fact columns per partition
  int32_t items;        // rows per consumer thread per tile
  uint64_t qvalid;      // bitmask of the batch's queries
  const DevCol* part_cols;   // [part][n_cols]
  const int64_t* tile_base;  // [n_parts + 1] first tile (kSBConsumerWarps * 32 * items rows) of each partition
  const int64_t* part_rows;  // [n_parts]
  int64_t n_tiles;
  int64_t tile_begin, tile_end;  // tiles of this launch
  const SBSegments* segs;        // [dimension]
  unsigned long long* gathered;  // rows that reached step (2), and step (3)
  uint64_t* gkeys;               // [gcap] group keys, shared by every query (all-ones = empty)
  unsigned long long* touched;   // [gcap + 1] queries with rows in each group; slot gcap: the all-ones key
  unsigned long long* gaccs;     // [q][gcap + 1][n_aggs]
  uint64_t gmask;                // gcap - 1
  int32_t staged;                // foreign-key columns are 16-byte aligned: tiles arrive by bulk copy
  int32_t stage_bytes;           // one pipeline stage: every foreign-key segment of a tile
  int32_t seg_off[kSBMaxDims];   // byte offset of dimension d's foreign keys in a stage
  int32_t fk_width[kSBMaxDims];  // 4 or 8
  int32_t masks_off;             // byte offset of the staged query masks in dynamic shared memory
  int32_t rings_off;             // byte offset of the consumer warps' rings in dynamic shared memory
  int32_t n_stages;              // stages in the foreign-key ring (2 to kSBMaxStages)
  int32_t pad2;
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

// Slot of a group key in the table shared by all queries (gmask + 1 for the
// all-ones key). A slot's key changes once, from empty to its final value, so
// a cached read that sees a key can trust it; one that sees empty is settled
// by the CAS.
__device__ __forceinline__ uint64_t sb_group_slot(const SBFactParams& p, uint64_t key) {
  if (key == kEmptySlot) return p.gmask + 1;
  uint64_t slot = hash_key(static_cast<int64_t>(key)) & p.gmask;
  for (uint64_t i = 0; i <= p.gmask; ++i) {
    uint64_t s = p.gkeys[slot];
    if (s == kEmptySlot)
      s = atomicCAS(reinterpret_cast<unsigned long long*>(p.gkeys + slot), static_cast<unsigned long long>(kEmptySlot),
                    static_cast<unsigned long long>(key));
    if (s == kEmptySlot || s == key) return slot;
    slot = (slot + 1) & p.gmask;
  }
  raise_status(p.st, GFPDB_ENOMEM, 120);
  return UINT64_MAX;
}

struct SBTile {
  int64_t start;  // first row within the partition
  int64_t rows;   // rows in this tile
  int part;
};

__device__ __forceinline__ SBTile sb_tile(const SBFactParams& p, int64_t tile, int64_t tile_rows, int* part) {
  while (*part + 1 < p.n_parts && p.tile_base[*part + 1] <= tile) ++*part;  // tiles only grow
  SBTile t;
  t.part = *part;
  t.start = (tile - p.tile_base[*part]) * tile_rows;
  const int64_t left = p.part_rows[*part] - t.start;
  t.rows = left < tile_rows ? left : tile_rows;
  return t;
}

// Bytes of dimension d's foreign keys that the bulk copy brings for a tile
// (a multiple of 16; the last few rows of a partition come by plain loads).
__device__ __forceinline__ uint32_t sb_seg_bytes(const SBFactParams& p, int d, int64_t rows) {
  return p.staged ? static_cast<uint32_t>((rows * p.fk_width[d]) & ~int64_t{15}) : 0u;
}

// Stage 2: one persistent pass over every tile of every partition.
// Warp kSBConsumerWarps is the producer: one lane streams each tile's
// foreign-key columns into a ring of p.n_stages shared-memory stages with
// cp.async.bulk, completing on the stage's "full" mbarrier. The other warps
// consume: each takes 32 * ITEMS rows of the tile (lanes on consecutive
// rows) and releases the stage on its "empty" mbarrier once it has read its
// foreign keys, so consumer warps drift apart instead of meeting at a block
// barrier.
//
// A consumer works in three steps, each with every lane busy:
//  (1) per row, the dimensions staged in shared memory: a byte per key (its
//      segment class) and the class -> query mask table, plus the group
//      values the dimension carries; the rows some query still wants are
//      appended (ballot + prefix) to the warp's first ring together with
//      their index into each direct dimension in global memory, so the ring
//      outlives the tile's stage;
//  (2) per 32 entries of that ring, those dimensions' lookups, all of an
//      entry's loads issued together; the surviving rows go to the warp's
//      second ring with their group key;
//  (3) per 32 entries of the second ring, the group slot (one probe of the
//      table shared by all queries), the measures, and one atomic add per
//      query and aggregate.
// Steps (2) and (3) wait for 32 entries, across tiles, so their memory
// round trips are paid once per 32 rows that need them, not once per tile.
// M is the query mask type: 32 bits for batches of at most 32 queries, else
// 64. Every wait is bounded: on timeout the kernel records GFPDB_ETIMEDOUT
// and stops.
constexpr int kSBRing = 64;     // entries of each per-warp ring (two chunks of 32)
constexpr int kSBRingDims = 2;  // direct dimensions whose lookups wait in ring 1
constexpr int kSBFastStaged = 3;  // staged dimensions the 32-bit fast path handles

template <typename M>
struct SBRings {
  // ring 1: rows that passed the staged dimensions, with their index into
  // each direct dimension still to look up (all-ones: key out of its range)
  uint32_t part1[kSBRing];
  uint32_t row1[kSBRing];
  M m1[kSBRing];
  uint32_t g1a[kSBRing], g1b[kSBRing];
  uint32_t idx1[kSBRingDims][kSBRing];
  // ring 2: surviving rows (partition, row) with their group key
  uint32_t part2[kSBRing];
  uint32_t row2[kSBRing];
  M m2[kSBRing];
  unsigned long long key2[kSBRing];
};

template <typename M>
__device__ __forceinline__ M sb_mask_cast(uint64_t v) {
  return static_cast<M>(v);
}

// The group key of a row from its group column values.
__device__ __forceinline__ uint64_t sb_group_key(int n_group, uint32_t g0, uint32_t g1) {
  return n_group == 1 ? static_cast<uint64_t>(g0) : n_group == 2 ? (static_cast<uint64_t>(g0) << 32) | g1 : 0ull;
}

template <typename M>
__device__ __forceinline__ int sb_ffs(M m) {
  return sizeof(M) == 8 ? __ffsll(static_cast<long long>(m)) : __ffs(static_cast<int>(m));
}

// Step (3) for the entries [head, head + n) of ring 2 (n <= 32), one per lane.
template <typename M>
__device__ __forceinline__ void sb_update_groups(const SBFactParams& p, SBRings<M>& R, uint32_t head, int n, int lane) {
  if (lane >= n) return;
  const uint32_t e = (head + lane) & (kSBRing - 1);
  M mi = R.m2[e];
  const int part = static_cast<int>(R.part2[e]);
  const int64_t row = R.row2[e];
  const DevCol* cols = p.part_cols + static_cast<int64_t>(part) * p.n_cols;
  unsigned long long vals[kSBMaxAggsFact];
#pragma unroll
  for (int a = 0; a < kSBMaxAggsFact; ++a) {
    vals[a] = 0;
    if (a >= p.n_aggs) continue;
    const SBAgg& g = p.aggs[a];
    if (g.fn == AGG_COUNT_STAR) {
      vals[a] = 1ull;
    } else {
      uint64_t x = static_cast<uint64_t>(load_int(cols[g.a], row));
      if (g.b >= 0) x *= static_cast<uint64_t>(load_int(cols[g.b], row));  // int64 wrap
      vals[a] = x;
    }
  }
  const uint64_t slot = sb_group_slot(p, R.key2[e]);
  if (slot == UINT64_MAX) return;
  atomicOr(p.touched + slot, static_cast<unsigned long long>(mi));
  while (mi != 0) {
    const int q = sb_ffs(mi) - 1;
    mi &= mi - 1;
    unsigned long long* acc =
        p.gaccs + (static_cast<uint64_t>(q) * (p.gmask + 2) + slot) * static_cast<uint64_t>(p.n_aggs);
#pragma unroll
    for (int a = 0; a < kSBMaxAggsFact; ++a)
      if (a < p.n_aggs) atomicAdd(acc + a, vals[a]);
  }
}

// The per-dimension facts a consumer reads per row, gathered once per block
// into shared memory in probe order: the dimensions staged in shared memory
// (step 1) and the direct dimensions in global memory (step 2).
struct SBStagedDim {
  int32_t d;        // dimension
  int32_t tab;      // byte offset of its class -> query mask table in the staged area
  int32_t cls;      // byte offset of its segment class per key
  int32_t seg;      // byte offset of its foreign keys in a stage
  int32_t w8;       // 8-byte foreign keys
  int32_t g0, g1;   // byte offsets of the values of group columns 0 / 1 it carries (-1: none)
  int32_t pad;
  int64_t kmin;
  uint64_t range;
};

struct SBGlobalDim {
  int32_t d;
  int32_t seg;
  int32_t w8;
  int32_t pad;
  int64_t kmin;
  uint64_t range;
  const uint64_t* dq;
  const int32_t* g0;  // group column 0 / 1 values by key - min (nullptr: not carried)
  const int32_t* g1;
};

// Step (2) for the entries [h1, h1 + n) of ring 1 (n <= 32), one per lane;
// survivors go to ring 2, which is worked off 32 entries at a time.
template <typename M, bool LOAD_FK = false>
__device__ __forceinline__ void sb_probe_global(const SBFactParams& p, SBRings<M>& R, const SBGlobalDim* gl, int nring,
                                             uint32_t h1, int n, uint32_t& h2, uint32_t& t2, int lane) {
  const uint32_t e1 = (h1 + lane) & (kSBRing - 1);
  M m = 0;
  uint32_t g0 = 0, g1 = 0, part = 0, row = 0;
  if (lane < n) {
    m = R.m1[e1];
    g0 = R.g1a[e1];
    g1 = R.g1b[e1];
    part = R.part1[e1];
    row = R.row1[e1];
  }
  uint64_t dq[kSBRingDims];
  uint32_t dg0[kSBRingDims], dg1[kSBRingDims];
#pragma unroll
  for (int u = 0; u < kSBRingDims; ++u) {
    dq[u] = ~0ull;
    dg0[u] = dg1[u] = 0;
    if (u >= nring || m == 0) continue;
    const SBGlobalDim& G = gl[u];
    uint32_t idx;
    if (LOAD_FK) {
      // the entry's foreign key of this dimension, read from its column
      // (int32 keys: the direct form)
      const int32_t fk =
          __ldg(static_cast<const int32_t*>(p.part_cols[static_cast<int64_t>(part) * p.n_cols + p.fd.fk_col[G.d]].data) +
                row);
      const uint64_t i64 = static_cast<uint64_t>(static_cast<int64_t>(fk) - G.kmin);
      idx = i64 < G.range ? static_cast<uint32_t>(i64) : 0xFFFFFFFFu;
    } else {
      idx = R.idx1[u][e1];
    }
    dq[u] = 0;
    if (idx != 0xFFFFFFFFu) {
      dq[u] = sizeof(M) == 4 ? static_cast<uint64_t>(__ldg(reinterpret_cast<const unsigned*>(G.dq) + 2 * idx))
                             : __ldg(reinterpret_cast<const unsigned long long*>(G.dq) + idx);
      if (G.g0 != nullptr) dg0[u] = static_cast<uint32_t>(__ldg(G.g0 + idx));
      if (G.g1 != nullptr) dg1[u] = static_cast<uint32_t>(__ldg(G.g1 + idx));
    }
  }
#pragma unroll
  for (int u = 0; u < kSBRingDims; ++u) {
    if (u >= nring) continue;
    m &= sb_mask_cast<M>(dq[u]);
    if (gl[u].g0 != nullptr) g0 = dg0[u];
    if (gl[u].g1 != nullptr) g1 = dg1[u];
  }
  const unsigned b = __ballot_sync(0xffffffffu, m != 0);
  if (m != 0) {
    const uint32_t e = (t2 + __popc(b & ((1u << lane) - 1u))) & (kSBRing - 1);
    R.part2[e] = part;
    R.row2[e] = row;
    R.m2[e] = m;
    R.key2[e] = sb_group_key(p.fd.n_group, g0, g1);
  }
  t2 += __popc(b);
  __syncwarp();
  if (t2 - h2 >= 32) {
    sb_update_groups<M>(p, R, h2, 32, lane);
    h2 += 32;
    __syncwarp();
  }
}

template <int ITEMS, typename M>
__global__ void __launch_bounds__(kSBFactThreads, 3) sb_fact_kernel(const __grid_constant__ SBFactParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + kSBMaxStages;
  unsigned char* stages = smem + kSBBarBytes;
  unsigned char* staged_dims = smem + p.masks_off;
  SBRings<M>* rings = reinterpret_cast<SBRings<M>*>(smem + p.rings_off);
  __shared__ int64_t s_kmin[kSBMaxDims];
  __shared__ uint64_t s_range[kSBMaxDims];
  __shared__ int32_t s_off[kSBMaxDims];  // staged: byte offset in staged_dims, else -1
  __shared__ SBStagedDim s_st[kSBMaxDims];
  __shared__ SBGlobalDim s_gl[kSBMaxDims];
  __shared__ int32_t s_nst, s_ngl, s_nhash;
  // The 32-bit fast path's facts (int32 keys, at most kSBFastStaged staged
  // dimensions): per staged dimension its foreign-key segment, smallest key,
  // key range, class table, classes and group values (byte offsets); per
  // ring dimension its segment, smallest key and range.
  __shared__ uint32_t s_fst[kSBFastStaged][8];
  __shared__ uint32_t s_frd[kSBRingDims][4];
  __shared__ int32_t s_fast;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < p.n_dims) {
    const SBDimDev& D = p.dims[threadIdx.x];
    const SBDirect dr = sb_direct(D);
    s_kmin[threadIdx.x] = dr.kmin;
    s_range[threadIdx.x] = dr.range;
    s_off[threadIdx.x] =
        (dr.range != 0 && D.smem_off >= 0 && dr.range <= static_cast<uint64_t>(D.smem_cap)) ? D.smem_off : -1;
  }
  uint64_t* staging = full + 2 * kSBMaxStages;
  if (threadIdx.x == 0) {
    for (int s = 0; s < p.n_stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kSBConsumerWarps);
    }
    mbar_init(staging, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const int gd0 = p.fd.n_group > 0 ? p.fd.group_dim[0] : -1;
  const int gd1 = p.fd.n_group > 1 ? p.fd.group_dim[1] : -1;
  if (threadIdx.x == 0) {
    int nst = 0, ngl = 0, nh = 0;
    for (int j = 0; j < p.n_dims; ++j) {
      const int d = p.fd.order[j];
      const SBDimDev& D = p.dims[d];
      if (s_off[d] >= 0) {
        // staged layout: the class -> mask table (256 masks), each group
        // column's values, then the classes (one byte per key)
        SBStagedDim& S = s_st[nst++];
        const int cap = D.smem_cap;
        const int tab = 256 * static_cast<int>(sizeof(M));
        S.d = d;
        S.tab = s_off[d];
        S.g0 = d == gd0 ? s_off[d] + tab + p.fd.group_idx[0] * cap * 4 : -1;
        S.g1 = d == gd1 ? s_off[d] + tab + p.fd.group_idx[1] * cap * 4 : -1;
        S.cls = s_off[d] + tab + D.n_group * cap * 4;
        S.seg = p.seg_off[d];
        S.w8 = p.fk_width[d] == 8;
        S.kmin = s_kmin[d];
        S.range = s_range[d];
      } else if (s_range[d] != 0) {
        SBGlobalDim& G = s_gl[ngl++];
        G.d = d;
        G.seg = p.seg_off[d];
        G.w8 = p.fk_width[d] == 8;
        G.kmin = s_kmin[d];
        G.range = s_range[d];
        G.dq = D.dq;
        G.g0 = d == gd0 ? D.dg[p.fd.group_idx[0]] : nullptr;
        G.g1 = d == gd1 ? D.dg[p.fd.group_idx[1]] : nullptr;
      } else {
        ++nh;
      }
    }
    s_nst = nst;
    s_ngl = ngl;
    s_nhash = nh;
    // fast path: int32 foreign keys and key ranges of every staged and ring
    // dimension, at most kSBFastStaged staged dimensions, no extra lookups
    bool fast = nst <= kSBFastStaged && ngl <= kSBRingDims && nh == 0;
    for (int j = 0; j < nst && fast; ++j) {
      const SBStagedDim& S = s_st[j];
      fast = !S.w8 && S.kmin >= INT32_MIN && S.kmin <= INT32_MAX && S.range <= (1ull << 31);
      uint32_t* f = s_fst[j];
      f[0] = static_cast<uint32_t>(S.seg);
      f[1] = static_cast<uint32_t>(static_cast<int32_t>(S.kmin));
      f[2] = static_cast<uint32_t>(S.range);
      f[3] = static_cast<uint32_t>(S.tab);
      f[4] = static_cast<uint32_t>(S.cls);
      f[5] = static_cast<uint32_t>(S.g0 >= 0 ? S.g0 : S.g1);  // the group column it carries, if any
      f[6] = S.g0 >= 0 ? 0u : S.g1 >= 0 ? 1u : 2u;              // which (2: none)
      f[7] = S.g0 >= 0 && S.g1 >= 0 ? static_cast<uint32_t>(S.g1) : 0xFFFFFFFFu;  // both: the second
    }
    for (int u = 0; u < ngl && fast; ++u) {
      const SBGlobalDim& G = s_gl[u];
      fast = !G.w8 && G.kmin >= INT32_MIN && G.kmin <= INT32_MAX && G.range <= (1ull << 31);
      s_frd[u][0] = static_cast<uint32_t>(G.seg);
      s_frd[u][1] = static_cast<uint32_t>(static_cast<int32_t>(G.kmin));
      s_frd[u][2] = static_cast<uint32_t>(G.range);
    }
    s_fast = fast ? 1 : 0;
  }
  // Staging: each staged dimension's classes and group values arrive by
  // bulk copies (16-byte multiples: the device arrays and the staged area
  // hold whole multiples of 16 keys), the class -> mask tables by loads.
  if (threadIdx.x == 0) {
    uint32_t bytes = 0;
    for (int d = 0; d < p.n_dims; ++d) {
      if (s_off[d] < 0) continue;
      const uint32_t keys = static_cast<uint32_t>((s_range[d] + 15) / 16 * 16);
      bytes += keys * (1 + 4 * p.dims[d].n_group);
    }
    mbar_arrive_expect_tx(staging, bytes);
    for (int d = 0; d < p.n_dims; ++d) {
      if (s_off[d] < 0) continue;
      const SBDimDev& D = p.dims[d];
      const int cap = D.smem_cap;
      const uint32_t keys = static_cast<uint32_t>((s_range[d] + 15) / 16 * 16);
      for (int c = 0; c < D.n_group; ++c)
        bulk_g2s(staged_dims + s_off[d] + 256 * sizeof(M) + c * cap * 4, D.dg[c], keys * 4, staging);
      bulk_g2s(staged_dims + s_off[d] + 256 * sizeof(M) + D.n_group * cap * 4, D.dclass, keys, staging);
    }
  }
  for (int d = 0; d < p.n_dims; ++d) {
    if (s_off[d] < 0) continue;
    M* tab = reinterpret_cast<M*>(staged_dims + s_off[d]);
    for (int i = threadIdx.x; i < 256; i += kSBFactThreads) tab[i] = sb_mask_cast<M>(p.segs[d].cmask[i]);
  }
  if (!mbar_wait(staging, 0)) raise_status(p.st, GFPDB_ETIMEDOUT, 133);
  __syncthreads();  // the last block-wide barrier: roles split below
  constexpr int64_t kTileRows = static_cast<int64_t>(kSBConsumerWarps) * 32 * ITEMS;
  int part = 0;
  if (warp == kSBConsumerWarps) {
    // ---------------------------------------------------------- producer
    if (lane != 0) return;
    int64_t k = 0;
    for (int64_t tile = p.tile_begin + blockIdx.x; tile < p.tile_end; tile += gridDim.x, ++k) {
      const int s = static_cast<int>(k % p.n_stages);
      if (k >= p.n_stages && !mbar_wait(&empty[s], static_cast<uint32_t>((k / p.n_stages - 1) & 1))) {
        raise_status(p.st, GFPDB_ETIMEDOUT, 130);
        break;
      }
      const SBTile t = sb_tile(p, tile, kTileRows, &part);
      const DevCol* cols = p.part_cols + static_cast<int64_t>(t.part) * p.n_cols;
      uint32_t bytes = 0;
      for (int d = 0; d < p.n_dims; ++d) bytes += sb_seg_bytes(p, d, t.rows);
      mbar_arrive_expect_tx(&full[s], bytes);
      for (int d = 0; d < p.n_dims; ++d) {
        const uint32_t b = sb_seg_bytes(p, d, t.rows);
        if (b == 0) continue;
        const unsigned char* src =
            static_cast<const unsigned char*>(cols[p.fd.fk_col[d]].data) + t.start * p.fk_width[d];
        bulk_g2s(stages + static_cast<int64_t>(s) * p.stage_bytes + p.seg_off[d], src, b, &full[s]);
      }
    }
    // Copies still in flight land before this CTA exits: wait for the
    // stages issued last (consumers wait on the same phases).
    const int64_t issued = k;
    for (int64_t j = issued > p.n_stages ? issued - p.n_stages : 0; j < issued; ++j)
      if (!mbar_wait(&full[j % p.n_stages], static_cast<uint32_t>((j / p.n_stages) & 1))) {
        raise_status(p.st, GFPDB_ETIMEDOUT, 131);
        break;
      }
    return;
  }
  // ------------------------------------------------------------ consumers
  SBRings<M>& R = rings[warp];
  const M qvalid = sb_mask_cast<M>(p.qvalid);
  const unsigned lt_mask = (1u << lane) - 1u;
  const int nst = s_nst, ngl = s_ngl, nhash = s_nhash;
  const int nring = ngl < kSBRingDims ? ngl : kSBRingDims;  // direct dimensions looked up in step (2)
  const bool fast = s_fast != 0;
  uint32_t h1 = 0, t1 = 0;  // ring 1 head / tail, kept across tiles
  uint32_t h2 = 0, t2 = 0;  // ring 2 head / tail
  int64_t k = 0;
  for (int64_t tile = p.tile_begin + blockIdx.x; tile < p.tile_end; tile += gridDim.x, ++k) {
    const int s = static_cast<int>(k % p.n_stages);
    const SBTile t = sb_tile(p, tile, kTileRows, &part);
    const DevCol* cols = p.part_cols + static_cast<int64_t>(t.part) * p.n_cols;
    const bool ok = mbar_wait(&full[s], static_cast<uint32_t>((k / p.n_stages) & 1));
    if (!__all_sync(0xffffffffu, ok)) {  // warp-uniform exit
      if (lane == 0) raise_status(p.st, GFPDB_ETIMEDOUT, 132);
      break;
    }
    const unsigned char* stage = stages + static_cast<int64_t>(s) * p.stage_bytes;
    // a full tile of a 16-byte-aligned partition is wholly in the stage
    const bool whole = p.staged && t.rows == kTileRows;
    // foreign key of dimension d for row r of the tile (stage or, for the
    // last rows of a partition, global memory)
    auto fk_of = [&](int d, int seg_off, bool w8, int64_t r) -> int64_t {
      const unsigned char* seg = stage + seg_off;
      if (whole || r < (static_cast<int64_t>(sb_seg_bytes(p, d, t.rows)) >> (w8 ? 3 : 2)))
        return w8 ? reinterpret_cast<const int64_t*>(seg)[r] : static_cast<int64_t>(reinterpret_cast<const int32_t*>(seg)[r]);
      return load_int(cols[p.fd.fk_col[d]], t.start + r);
    };
    if (fast && whole) {
      // 32-bit fast path: the whole tile is in the stage, keys are int32
#pragma unroll 1
      for (int i = 0; i < ITEMS; ++i) {
        const uint32_t r = static_cast<uint32_t>(warp * 32 * ITEMS + i * 32 + lane);
        M m = qvalid;
        uint32_t g0 = 0, g1 = 0;
#pragma unroll
        for (int j = 0; j < kSBFastStaged; ++j) {
          if (j >= nst || m == 0) continue;
          const uint32_t* f = s_fst[j];
          const int32_t fk = reinterpret_cast<const int32_t*>(stage + f[0])[r];
          const int32_t kmin = static_cast<int32_t>(f[1]);
          const uint32_t idx = static_cast<uint32_t>(fk) - static_cast<uint32_t>(kmin);
          M q = 0;
          if (fk >= kmin && idx < f[2]) q = reinterpret_cast<const M*>(staged_dims + f[3])[staged_dims[f[4] + idx]];
          m &= q;
          if (m != 0 && f[6] != 2u) {
            const uint32_t gv = reinterpret_cast<const uint32_t*>(staged_dims + f[5])[idx];
            if (f[6] == 0u) g0 = gv;
            else g1 = gv;
            if (f[7] != 0xFFFFFFFFu) g1 = reinterpret_cast<const uint32_t*>(staged_dims + f[7])[idx];
          }
        }
        const unsigned b = __ballot_sync(0xffffffffu, m != 0);
        if (m != 0) {
          const uint32_t e = (t1 + __popc(b & lt_mask)) & (kSBRing - 1);
          R.part1[e] = static_cast<uint32_t>(t.part);
          R.row1[e] = static_cast<uint32_t>(t.start) + r;
          R.m1[e] = m;
          R.g1a[e] = g0;
          R.g1b[e] = g1;
#pragma unroll
          for (int u = 0; u < kSBRingDims; ++u) {
            if (u >= nring) continue;
            const int32_t fk = reinterpret_cast<const int32_t*>(stage + s_frd[u][0])[r];
            const int32_t kmin = static_cast<int32_t>(s_frd[u][1]);
            const uint32_t idx = static_cast<uint32_t>(fk) - static_cast<uint32_t>(kmin);
            R.idx1[u][e] = fk >= kmin && idx < s_frd[u][2] ? idx : 0xFFFFFFFFu;
          }
        }
        t1 += __popc(b);
        __syncwarp();
        if (t1 - h1 >= 32) {
          sb_probe_global<M>(p, R, s_gl, nring, h1, 32, h2, t2, lane);
          h1 += 32;
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      continue;
    }
#pragma unroll 1
    for (int i = 0; i < ITEMS; ++i) {
      const int64_t r = static_cast<int64_t>(warp) * 32 * ITEMS + i * 32 + lane;  // row within the tile
      M m = r < t.rows ? qvalid : M(0);
      uint32_t g0 = 0, g1 = 0;
      // Step (1): dimensions staged in shared memory, in probe order
      for (int j = 0; j < nst; ++j) {
        const SBStagedDim& S = s_st[j];
        if (m != 0) {
          const uint64_t idx = static_cast<uint64_t>(fk_of(S.d, S.seg, S.w8, r)) - static_cast<uint64_t>(S.kmin);
          m &= idx < S.range ? reinterpret_cast<const M*>(staged_dims + S.tab)[staged_dims[S.cls + idx]] : M(0);
          if (m != 0 && S.g0 >= 0) g0 = reinterpret_cast<const uint32_t*>(staged_dims + S.g0)[idx];
          if (m != 0 && S.g1 >= 0) g1 = reinterpret_cast<const uint32_t*>(staged_dims + S.g1)[idx];
        }
      }
      // direct dimensions past the ring's kSBRingDims, and dimensions looked
      // up by hash (sparse keys): per row, here
      for (int j = nring; m != 0 && j < ngl + (nhash > 0 ? p.n_dims : 0); ++j) {
        const bool hashed = j >= ngl;
        const int d = hashed ? j - ngl : s_gl[j].d;
        if (hashed && s_range[d] != 0) continue;
        const SBDimDev& D = p.dims[d];
        const int64_t key = fk_of(d, p.seg_off[d], p.fk_width[d] == 8, r);
        int64_t dr = -1;
        M q = 0;
        if (hashed) {
          dr = sb_lookup(D, key);
          if (dr >= 0) q = sb_mask_cast<M>(__ldg(reinterpret_cast<const unsigned long long*>(D.qmask + dr)));
        } else {
          const uint64_t idx = static_cast<uint64_t>(key) - static_cast<uint64_t>(s_kmin[d]);
          if (idx < s_range[d]) {
            q = sb_mask_cast<M>(__ldg(reinterpret_cast<const unsigned long long*>(D.dq + idx)));
            dr = static_cast<int64_t>(idx);
          }
        }
        m &= q;
        if (m != 0 && d == gd0)
          g0 = static_cast<uint32_t>(hashed ? load_int(D.group[p.fd.group_idx[0]], dr) : __ldg(D.dg[p.fd.group_idx[0]] + dr));
        if (m != 0 && d == gd1)
          g1 = static_cast<uint32_t>(hashed ? load_int(D.group[p.fd.group_idx[1]], dr) : __ldg(D.dg[p.fd.group_idx[1]] + dr));
      }
      const unsigned b = __ballot_sync(0xffffffffu, m != 0);
      if (m != 0) {
        const uint32_t e = (t1 + __popc(b & lt_mask)) & (kSBRing - 1);
        R.part1[e] = static_cast<uint32_t>(t.part);
        R.row1[e] = static_cast<uint32_t>(t.start + r);
        R.m1[e] = m;
        R.g1a[e] = g0;
        R.g1b[e] = g1;
        for (int u = 0; u < nring; ++u) {
          const SBGlobalDim& G = s_gl[u];
          const uint64_t idx = static_cast<uint64_t>(fk_of(G.d, G.seg, G.w8, r)) - static_cast<uint64_t>(G.kmin);
          R.idx1[u][e] = idx < G.range ? static_cast<uint32_t>(idx) : 0xFFFFFFFFu;
        }
      }
      t1 += __popc(b);
      __syncwarp();
      if (t1 - h1 >= 32) {
        sb_probe_global<M>(p, R, s_gl, nring, h1, 32, h2, t2, lane);
        h1 += 32;
      }
    }
    // Every foreign key this warp needs from the stage has been read.
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  // the warp's last rows: ring 1, then ring 2
  while (t1 != h1) {
    const int n = t1 - h1 < 32 ? static_cast<int>(t1 - h1) : 32;
    sb_probe_global<M>(p, R, s_gl, nring, h1, n, h2, t2, lane);
    h1 += n;
  }
  while (t2 != h2) {
    const int n = t2 - h2 < 32 ? static_cast<int>(t2 - h2) : 32;
    sb_update_groups<M>(p, R, h2, n, lane);
    h2 += n;
    __syncwarp();
  }
  if (lane == 0) {
    atomicAdd(p.gathered, static_cast<unsigned long long>(t1));
    atomicAdd(p.gathered + 1, static_cast<unsigned long long>(t2));
  }
}

// Stage 2, direct form: for int32 foreign and dimension keys in 16-byte
// aligned columns. Every warp takes whole tiles (256 * ITEMS rows) in turn
// and reads each 128-row slice of a tile itself, four consecutive rows per
// lane by 16-byte loads: no producer warp, no copy stages and no waits
// between warps, so the shared memory goes to the staged dimensions (up to
// kSBFastStaged of them) and the rings, and each block stages them once for
// all its warps. Steps (1)-(3) are those of sb_fact_kernel; step (1) runs
// in 32-bit arithmetic on the lane's four rows.
constexpr int kSBDirectWarps = 16;
constexpr int kSBDirectThreads = kSBDirectWarps * 32;
constexpr int kSBSlice = 128;  // rows per warp step: four per lane

struct SBShared {
  int64_t kmin[kSBMaxDims];
  uint64_t range[kSBMaxDims];
  int32_t off[kSBMaxDims];  // staged: byte offset in the staged area, else -1
  SBGlobalDim gl[kSBMaxDims];
  // staged dimensions in probe order: foreign-key column slot, smallest key,
  // key range, class table, classes, group value offsets (-1: none)
  int32_t st_col[kSBFastStaged];
  int32_t st_kmin[kSBFastStaged];
  uint32_t st_range[kSBFastStaged];
  int32_t st_tab[kSBFastStaged], st_cls[kSBFastStaged], st_g0[kSBFastStaged], st_g1[kSBFastStaged];
  int32_t nst, ngl, nhash;
};

// Step (1)'s lookups of a row in the dimensions the direct form cannot
// stage or ring: direct dimensions past the ring's kSBRingDims, and
// dimensions looked up by hash (sparse keys).
template <typename M>
__device__ __forceinline__ void sb_extra_lookups(const SBFactParams& p, const SBShared& sh, const DevCol* cols, int64_t row,
                                              int nring, M& m, uint32_t& g0, uint32_t& g1) {
  const int gd0 = p.fd.n_group > 0 ? p.fd.group_dim[0] : -1;
  const int gd1 = p.fd.n_group > 1 ? p.fd.group_dim[1] : -1;
  for (int j = nring; m != 0 && j < sh.ngl + (sh.nhash > 0 ? p.n_dims : 0); ++j) {
    const bool hashed = j >= sh.ngl;
    const int d = hashed ? j - sh.ngl : sh.gl[j].d;
    if (hashed && sh.range[d] != 0) continue;
    const SBDimDev& D = p.dims[d];
    const int64_t key = load_int(cols[p.fd.fk_col[d]], row);
    int64_t dr = -1;
    M q = 0;
    if (hashed) {
      dr = sb_lookup(D, key);
      if (dr >= 0) q = sb_mask_cast<M>(__ldg(reinterpret_cast<const unsigned long long*>(D.qmask + dr)));
    } else {
      const uint64_t idx = static_cast<uint64_t>(key) - static_cast<uint64_t>(sh.kmin[d]);
      if (idx < sh.range[d]) {
        q = sb_mask_cast<M>(__ldg(reinterpret_cast<const unsigned long long*>(D.dq + idx)));
        dr = static_cast<int64_t>(idx);
      }
    }
    m &= q;
    if (m != 0 && d == gd0)
      g0 = static_cast<uint32_t>(hashed ? load_int(D.group[p.fd.group_idx[0]], dr) : __ldg(D.dg[p.fd.group_idx[0]] + dr));
    if (m != 0 && d == gd1)
      g1 = static_cast<uint32_t>(hashed ? load_int(D.group[p.fd.group_idx[1]], dr) : __ldg(D.dg[p.fd.group_idx[1]] + dr));
  }
}

template <int ITEMS, typename M>
__global__ void __launch_bounds__(kSBDirectThreads, 2) sb_fact_direct_kernel(const __grid_constant__ SBFactParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t staging;
  __shared__ SBShared sh;
  unsigned char* staged_dims = smem + p.masks_off;
  SBRings<M>* rings = reinterpret_cast<SBRings<M>*>(smem + p.rings_off);
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int gd0 = p.fd.n_group > 0 ? p.fd.group_dim[0] : -1;
  const int gd1 = p.fd.n_group > 1 ? p.fd.group_dim[1] : -1;
  if (threadIdx.x < p.n_dims) {
    const SBDimDev& D = p.dims[threadIdx.x];
    const SBDirect dr = sb_direct(D);
    sh.kmin[threadIdx.x] = dr.kmin;
    sh.range[threadIdx.x] = dr.range;
    sh.off[threadIdx.x] =
        (dr.range != 0 && D.smem_off >= 0 && dr.range <= static_cast<uint64_t>(D.smem_cap)) ? D.smem_off : -1;
  }
  if (threadIdx.x == 0) {
    mbar_init(&staging, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nst = 0, ngl = 0, nh = 0;
    uint32_t bytes = 0;
    for (int j = 0; j < p.n_dims; ++j) {
      const int d = p.fd.order[j];
      const SBDimDev& D = p.dims[d];
      if (sh.off[d] >= 0 && nst < kSBFastStaged) {
        // staged layout: the class -> mask table (256 masks), each group
        // column's values, then the classes (one byte per key)
        const int cap = D.smem_cap;
        const int tab = 256 * static_cast<int>(sizeof(M));
        const int o = sh.off[d];
        sh.st_col[nst] = p.fd.fk_col[d];
        sh.st_kmin[nst] = static_cast<int32_t>(sh.kmin[d]);
        sh.st_range[nst] = static_cast<uint32_t>(sh.range[d]);
        sh.st_tab[nst] = o;
        sh.st_g0[nst] = d == gd0 ? o + tab + p.fd.group_idx[0] * cap * 4 : -1;
        sh.st_g1[nst] = d == gd1 ? o + tab + p.fd.group_idx[1] * cap * 4 : -1;
        sh.st_cls[nst] = o + tab + D.n_group * cap * 4;
        const uint32_t keys = static_cast<uint32_t>((sh.range[d] + 15) / 16 * 16);
        bytes += keys * (1 + 4 * D.n_group);
        ++nst;
      } else if (sh.range[d] != 0) {
        sh.off[d] = -1;  // looked up in global memory
        SBGlobalDim& G = sh.gl[ngl];
        G.d = d;
        G.seg = 0;
        G.w8 = 0;
        G.kmin = sh.kmin[d];
        G.range = sh.range[d];
        G.dq = D.dq;
        G.g0 = d == gd0 ? D.dg[p.fd.group_idx[0]] : nullptr;
        G.g1 = d == gd1 ? D.dg[p.fd.group_idx[1]] : nullptr;
        ++ngl;
      } else {
        ++nh;
      }
    }
    sh.nst = nst;
    sh.ngl = ngl;
    sh.nhash = nh;
    // classes and group values of the staged dimensions by bulk copies
    // (16-byte multiples: the device arrays and the staged area hold whole
    // multiples of 16 keys)
    mbar_arrive_expect_tx(&staging, bytes);
    for (int j = 0; j < p.n_dims; ++j) {
      const int d = p.fd.order[j];
      if (sh.off[d] < 0) continue;
      const SBDimDev& D = p.dims[d];
      const int cap = D.smem_cap;
      const uint32_t keys = static_cast<uint32_t>((sh.range[d] + 15) / 16 * 16);
      for (int c = 0; c < D.n_group; ++c)
        bulk_g2s(staged_dims + sh.off[d] + 256 * sizeof(M) + c * cap * 4, D.dg[c], keys * 4, &staging);
      bulk_g2s(staged_dims + sh.off[d] + 256 * sizeof(M) + D.n_group * cap * 4, D.dclass, keys, &staging);
    }
  }
  __syncthreads();
  for (int d = 0; d < p.n_dims; ++d) {
    if (sh.off[d] < 0) continue;
    M* tab = reinterpret_cast<M*>(staged_dims + sh.off[d]);
    for (int i = threadIdx.x; i < 256; i += kSBDirectThreads) tab[i] = sb_mask_cast<M>(p.segs[d].cmask[i]);
  }
  if (!mbar_wait(&staging, 0)) raise_status(p.st, GFPDB_ETIMEDOUT, 134);
  __syncthreads();

  SBRings<M>& R = rings[warp];
  const M qvalid = sb_mask_cast<M>(p.qvalid);
  const unsigned lt_mask = (1u << lane) - 1u;
  const int nst = sh.nst, ngl = sh.ngl, nhash = sh.nhash;
  const int nring = ngl < kSBRingDims ? ngl : kSBRingDims;
  const bool extra = ngl > nring || nhash > 0;  // lookups step (1) makes per row
  uint32_t h1 = 0, t1 = 0, h2 = 0, t2 = 0;
  constexpr int64_t kTileRows = static_cast<int64_t>(kSBConsumerWarps) * 32 * ITEMS;
  int part = 0;
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * kSBDirectWarps;
  for (int64_t tile = p.tile_begin + static_cast<int64_t>(blockIdx.x) * kSBDirectWarps + warp; tile < p.tile_end;
       tile += nwarps) {
    const SBTile t = sb_tile(p, tile, kTileRows, &part);
    const DevCol* cols = p.part_cols + static_cast<int64_t>(t.part) * p.n_cols;
    for (int64_t sub = 0; sub < t.rows; sub += kSBSlice) {
      const int64_t row0 = t.start + sub;  // the slice's first row in the partition
      const int nrows = t.rows - sub < kSBSlice ? static_cast<int>(t.rows - sub) : kSBSlice;
      const int r4 = lane * 4;  // the lane's first row in the slice
      // foreign keys of the lane's four rows: staged and ring dimensions
      int4 fs[kSBFastStaged];
      auto load4 = [&](int col) -> int4 {
        const int32_t* c = static_cast<const int32_t*>(cols[col].data) + row0 + r4;
        if (nrows == kSBSlice) return __ldg(reinterpret_cast<const int4*>(c));
        int4 v = make_int4(0, 0, 0, 0);
        if (r4 + 0 < nrows) v.x = __ldg(c + 0);
        if (r4 + 1 < nrows) v.y = __ldg(c + 1);
        if (r4 + 2 < nrows) v.z = __ldg(c + 2);
        if (r4 + 3 < nrows) v.w = __ldg(c + 3);
        return v;
      };
#pragma unroll
      for (int j = 0; j < kSBFastStaged; ++j) fs[j] = j < nst ? load4(sh.st_col[j]) : make_int4(0, 0, 0, 0);
      // Step (1): the staged dimensions in probe order, each one's facts
      // read once for the lane's four rows
      M mk[4];
      uint32_t g0k[4], g1k[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        mk[k] = r4 + k < nrows ? qvalid : M(0);
        g0k[k] = g1k[k] = 0;
      }
#pragma unroll
      for (int j = 0; j < kSBFastStaged; ++j) {
        if (j >= nst) break;
        const int32_t kmin = sh.st_kmin[j];
        const uint32_t range = sh.st_range[j];
        const M* tab = reinterpret_cast<const M*>(staged_dims + sh.st_tab[j]);
        const uint8_t* cls = staged_dims + sh.st_cls[j];
        const int go0 = sh.st_g0[j], go1 = sh.st_g1[j];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int32_t fk = k == 0 ? fs[j].x : k == 1 ? fs[j].y : k == 2 ? fs[j].z : fs[j].w;
          const uint32_t idx = static_cast<uint32_t>(fk) - static_cast<uint32_t>(kmin);
          const bool in = mk[k] != 0 && fk >= kmin && idx < range;
          mk[k] = in ? mk[k] & tab[cls[idx]] : M(0);
          if (mk[k] != 0 && go0 >= 0) g0k[k] = reinterpret_cast<const uint32_t*>(staged_dims + go0)[idx];
          if (mk[k] != 0 && go1 >= 0) g1k[k] = reinterpret_cast<const uint32_t*>(staged_dims + go1)[idx];
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int rin = r4 + k;
        M m = mk[k];
        uint32_t g0 = g0k[k], g1 = g1k[k];
        // direct dimensions past the ring's, and dimensions looked up by
        // hash (sparse keys): per row, out of line
        if (extra && m != 0) sb_extra_lookups<M>(p, sh, cols, row0 + rin, nring, m, g0, g1);
        const unsigned b = __ballot_sync(0xffffffffu, m != 0);
        if (m != 0) {
          const uint32_t e = (t1 + __popc(b & lt_mask)) & (kSBRing - 1);
          R.part1[e] = static_cast<uint32_t>(t.part);
          R.row1[e] = static_cast<uint32_t>(row0 + rin);
          R.m1[e] = m;
          R.g1a[e] = g0;
          R.g1b[e] = g1;
        }
        t1 += __popc(b);
        __syncwarp();
        if (t1 - h1 >= 32) {
          sb_probe_global<M, true>(p, R, sh.gl, nring, h1, 32, h2, t2, lane);
          h1 += 32;
        }
      }
    }
  }
  // the warp's last rows: ring 1, then ring 2
  while (t1 != h1) {
    const int n = t1 - h1 < 32 ? static_cast<int>(t1 - h1) : 32;
    sb_probe_global<M, true>(p, R, sh.gl, nring, h1, n, h2, t2, lane);
    h1 += n;
  }
  while (t2 != h2) {
    const int n = t2 - h2 < 32 ? static_cast<int>(t2 - h2) : 32;
    sb_update_groups<M>(p, R, h2, n, lane);
    h2 += n;
    __syncwarp();
  }
  if (lane == 0) {
    atomicAdd(p.gathered, static_cast<unsigned long long>(t1));
    atomicAdd(p.gathered + 1, static_cast<unsigned long long>(t2));
  }
}

struct SBFinalParams {
  const uint64_t* gkeys;
  const unsigned long long* touched;
  const unsigned long long* gaccs;
  uint64_t slots;  // gcap + 1
  int32_t n_queries;
  int32_t n_aggs;
  int32_t n_group;
  int32_t pad;
  int32_t* out_q;
  void* out_g[2];
  long long* out_a[kMaxAggs];
  unsigned long long* counter;   // output rows in all
  unsigned long long* qcount;    // [kSBMaxQueries] output rows of each query
  unsigned long long* qcursor;   // [kSBMaxQueries]
  unsigned long long* qoff;      // [kSBMaxQueries + 1] first output row of each query
};

// Stage 3a: output rows of each query (groups it touched).
__global__ void __launch_bounds__(256) sb_count_kernel(const __grid_constant__ SBFinalParams p) {
  __shared__ unsigned int s_cnt[kSBMaxQueries];
  for (int q = threadIdx.x; q < kSBMaxQueries; q += blockDim.x) s_cnt[q] = 0;
  __syncthreads();
  for (uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; s < p.slots;
       s += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    unsigned long long m = p.touched[s];
    while (m != 0) {
      atomicAdd(&s_cnt[__ffsll(static_cast<long long>(m)) - 1], 1u);
      m &= m - 1;
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kSBMaxQueries; q += blockDim.x)
    if (s_cnt[q] != 0) atomicAdd(p.qcount + q, static_cast<unsigned long long>(s_cnt[q]));
}

// Stage 3b: every (query, group) with rows becomes one output row; each
// query's rows are contiguous (queries in order), so a query's result is a
// slice of the output.
__global__ void __launch_bounds__(256) sb_final_kernel(const __grid_constant__ SBFinalParams p) {
  __shared__ unsigned long long s_off[kSBMaxQueries];
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int q = 0; q < kSBMaxQueries; ++q) {
      s_off[q] = acc;
      acc += p.qcount[q];
    }
    if (blockIdx.x == 0) {
      for (int q = 0; q < kSBMaxQueries; ++q) p.qoff[q] = s_off[q];
      p.qoff[kSBMaxQueries] = acc;
      *p.counter = acc;
    }
  }
  __syncthreads();
  const uint64_t total = p.slots * static_cast<uint64_t>(p.n_queries);
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const int q = static_cast<int>(i / p.slots);
    const uint64_t s = i % p.slots;
    if (((p.touched[s] >> q) & 1ull) == 0) continue;
    const uint64_t key = s + 1 < p.slots ? p.gkeys[s] : kEmptySlot;
    const int64_t pos = static_cast<int64_t>(s_off[q] + atomicAdd(p.qcursor + q, 1ull));
    p.out_q[pos] = q;
    if (p.n_group == 1) {
      static_cast<int32_t*>(p.out_g[0])[pos] = static_cast<int32_t>(static_cast<uint32_t>(key));
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

// Segments of every dimension from the queries' ranges (query q, dimension
// d: lo <= value <= hi; an empty range selects nothing).
static void fill_segments(const std::vector<std::vector<std::pair<int64_t, int64_t>>>& queries, int nd,
                          SBSegments* out) {
  for (int d = 0; d < nd; ++d) {
    SBSegments& S = out[d];
    std::memset(&S, 0, sizeof(S));
    std::vector<int64_t> b;
    for (const auto& q : queries) {
      const int64_t lo = q[d].first, hi = q[d].second;
      if (lo > hi) continue;
      b.push_back(lo);
      if (hi != INT64_MAX) b.push_back(hi + 1);
    }
    std::sort(b.begin(), b.end());
    b.erase(std::unique(b.begin(), b.end()), b.end());
    S.n_bounds = static_cast<int64_t>(b.size());  // at most 2 per query
    for (size_t i = 0; i < b.size(); ++i) S.bounds[i] = b[i];
    // segment k holds the values v with b[k - 1] <= v < b[k]; segment 0
    // (below every lo) and the last (from the last hi + 1 on) select nothing
    for (size_t k = 1; k <= b.size(); ++k) {
      const int64_t v = b[k - 1];  // every value of segment k is selected like this one
      unsigned long long m = 0;
      for (size_t qi = 0; qi < queries.size(); ++qi)
        if (queries[qi][d].first <= v && v <= queries[qi][d].second) m |= 1ull << qi;
      S.cmask[k] = m;
    }
    S.cmask[kSBNoRow] = 0;
  }
}

struct StarBatchState {
  StarBatchSpec spec;
  std::vector<TupleSetPtr> parts, dim_tables;
  std::vector<std::string> fact_cols;
  SBDimsParams dims_params;
  SBFactParams fact_params;
  BufferPtr tables_buf, masks_buf, dq_buf, drow_buf, dg_buf, dclass_buf, krange_buf, gkeys_buf, touched_buf, gaccs_buf, misc_buf, meta_buf,
      out_q;
  BufferPtr out_g[2], out_a[kMaxAggs];
  size_t fact_smem = 0;  // dynamic shared memory of a fact-stage block
  int mask_bytes = 8;    // query mask width in the fact stage (4: at most 32 queries)
  bool direct = false;   // the fact stage runs sb_fact_direct_kernel
  std::vector<char> host_meta;
  DType group_types[2] = {DType::Int32, DType::Int32};
  uint64_t gcap = 0;
  int64_t out_cap = 0, n_tiles = 0, fact_rows = 0;
  unsigned long long* counter = nullptr;
  unsigned long long* qcount = nullptr;
  unsigned long long* qcursor = nullptr;
  unsigned long long* qoff = nullptr;
  size_t ranges_host_off = 0;  // byte offset of the query ranges in host_meta / meta_buf
  // host-resident inputs
  struct Copy {
    void* dst;
    const void* src;
    int64_t bytes;
  };
  std::vector<StarBatchHostColumn> host_cols;
  std::vector<Copy> dim_copies;
  std::vector<std::vector<Copy>> group_copies;  // per group of partitions
  struct TileGroup {
    int64_t begin, end, rows;
  };
  std::vector<TileGroup> group_tiles;
  int64_t host_bytes = 0;
  std::vector<char> in_place;       // per fact column: read in place from page-locked host memory
  int n_in_place_fk = 0, n_in_place_measures = 0;
  unsigned long long* gathered = nullptr;
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> events;  // start, dimensions, then one per group

  ~StarBatchState();
  void plan_host_copies();

  void prepare(cudaStream_t s);
  void run(cudaStream_t s);
  void launch_fact(int grid, cudaStream_t s);
  TupleSetPtr result_view() const;
  const DevStatus* status() const;
  void set_ranges(const std::vector<std::vector<std::pair<int64_t, int64_t>>>& q, cudaStream_t s);
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
void StarBatch::set_ranges(const std::vector<std::vector<std::pair<int64_t, int64_t>>>& q, cudaStream_t s) {
  st_->set_ranges(q, s);
}
const unsigned long long* StarBatch::query_offsets() const { return st_->qoff; }
void StarBatch::set_host_columns(std::vector<StarBatchHostColumn> cols) { st_->host_cols = std::move(cols); }
int64_t StarBatch::host_bytes() const { return st_->host_bytes; }
const unsigned long long* StarBatch::gathered() const { return st_->gathered; }
int64_t StarBatch::in_place_bytes(uint64_t ring_rows, uint64_t survivor_rows) const {
  // one 32-byte sector per row and column read in place (an upper bound:
  // rows that share a sector are counted once each)
  return static_cast<int64_t>(32 * (ring_rows * st_->n_in_place_fk + survivor_rows * st_->n_in_place_measures));
}

StarBatchState::~StarBatchState() {
  for (cudaEvent_t e : events) (void)cudaEventDestroy(e);
  if (copy_stream != nullptr) (void)cudaStreamDestroy(copy_stream);
}

// Which host columns each run copies, and in which order: the dimensions'
// key, filter and group columns first, then the fact columns partition by
// partition in up to kSBCopyGroups groups of about equal rows; the fact pass
// runs once per group, after that group's copies.
constexpr int kSBCopyGroups = 8;

void StarBatchState::plan_host_copies() {
  dim_copies.clear();
  group_copies.clear();
  group_tiles.clear();
  host_bytes = 0;
  if (host_cols.empty()) return;
  auto add = [&](std::vector<Copy>& out, const void* dst, int64_t bytes) {
    if (bytes <= 0) return;
    for (const Copy& c : out)
      if (c.dst == dst) return;  // a column used twice is copied once
    for (const auto& h : host_cols)
      if (h.dst == dst && h.bytes >= bytes) {
        out.push_back(Copy{const_cast<void*>(dst), h.src, bytes});
        host_bytes += bytes;
        return;
      }
    // not in the list: the column is device-resident
  };
  for (size_t d = 0; d < dim_tables.size(); ++d) {
    const TupleSet& t = *dim_tables[d];
    const auto& ds = spec.dims[d];
    const int64_t n = t.num_rows();
    for (const std::string& c : {ds.key, ds.filter}) {
      const auto& col = t.column(c);
      add(dim_copies, col->data, n * dtype_width(col->type));
    }
    for (const auto& g : spec.group)
      if (g.dim == static_cast<int>(d)) {
        const auto& col = t.column(g.column);
        add(dim_copies, col->data, n * dtype_width(col->type));
      }
  }
  const int groups = static_cast<int>(std::min<size_t>(kSBCopyGroups, parts.size()));
  const int64_t tile_rows = static_cast<int64_t>(kSBConsumerWarps) * 32 * spec.items_per_thread;
  int64_t tiles = 0, rows_done = 0;
  size_t pi = 0;
  for (int g = 0; g < groups; ++g) {
    std::vector<Copy> cs;
    const int64_t tile_begin = tiles, rows_begin = rows_done;
    const int64_t target = fact_rows * (g + 1) / groups;
    while (pi < parts.size() && (rows_done < target || g == groups - 1)) {
      const TupleSet& t = *parts[pi];
      for (size_t c = 0; c < fact_cols.size(); ++c) {
        if (!in_place.empty() && in_place[c]) continue;
        const auto& col = t.column(fact_cols[c]);
        add(cs, col->data, t.num_rows() * dtype_width(col->type));
      }
      rows_done += t.num_rows();
      tiles += (t.num_rows() + tile_rows - 1) / tile_rows;
      ++pi;
    }
    if (tiles == tile_begin && cs.empty()) continue;
    group_copies.push_back(std::move(cs));
    group_tiles.push_back(TileGroup{tile_begin, tiles, rows_done - rows_begin});
  }
  if (copy_stream == nullptr) GF_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
  while (events.size() < group_copies.size() + 2) {
    cudaEvent_t e = nullptr;
    GF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    events.push_back(e);
  }
}

void StarBatchState::prepare(cudaStream_t s) {
  if (spec.dims.empty() || spec.dims.size() > static_cast<size_t>(kSBMaxDims))
    fail(GFPDB_EUNSUPPORTED, "a batched star query needs 1 to 8 dimensions");
  if (spec.queries.empty() || spec.queries.size() > static_cast<size_t>(kSBMaxQueries))
    fail(GFPDB_EUNSUPPORTED, "a batch holds 1 to 64 queries");
  if (spec.group.size() > 2) fail(GFPDB_EUNSUPPORTED, "at most two group columns in a batched star query");
  if (spec.aggs.empty() || spec.aggs.size() > static_cast<size_t>(kSBMaxAggsFact))
    fail(GFPDB_EUNSUPPORTED, "1 to 4 aggregates in a batched star query");
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
  if (items != 1 && items != 2 && items != 4 && items != 8)
    fail(GFPDB_EINVAL, "itemsPerThread must be 1, 2, 4 or 8");
  const int64_t tile_rows = static_cast<int64_t>(kSBConsumerWarps) * 32 * items;
  std::vector<int32_t> fk_width(nd, 0);
  bool aligned = true;
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
    for (int d = 0; d < nd; ++d) {
      const auto& col = t.column(fact_cols[fk_slot[d]]);
      const int32_t w = col->type == DType::Int64 ? 8 : 4;
      if (fk_width[d] != 0 && fk_width[d] != w)
        fail(GFPDB_EUNSUPPORTED, "batched star partitions must agree on foreign-key column types");
      fk_width[d] = w;
      aligned &= reinterpret_cast<uintptr_t>(col->data) % 16 == 0;
    }
    if (t.num_rows() > static_cast<int64_t>(UINT32_MAX))
      fail(GFPDB_EUNSUPPORTED, "a batched star partition holds at most 4,294,967,295 rows");
    hbase[pi] = tiles;
    hrows[pi] = t.num_rows();
    tiles += (t.num_rows() + tile_rows - 1) / tile_rows;
    fact_rows += t.num_rows();
  }
  hbase[parts.size()] = tiles;
  n_tiles = tiles;
  // pipeline stage: the tile's foreign keys of every dimension, one segment each
  std::memset(&fact_params, 0, sizeof(fact_params));
  int64_t stage_bytes = 0;
  for (int d = 0; d < nd; ++d) {
    fact_params.seg_off[d] = static_cast<int32_t>(stage_bytes);
    fact_params.fk_width[d] = fk_width[d];
    stage_bytes += tile_rows * fk_width[d];  // tile_rows is a multiple of 256: segments stay 16-byte aligned
  }
  fact_params.staged = aligned ? 1 : 0;
  fact_params.stage_bytes = static_cast<int32_t>(stage_bytes);
  fact_params.n_stages = spec.stages;
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
  // Shared-memory staging: the smallest dimensions first, one 64-bit mask
  // per key, within a per-block budget that leaves room for blocks_per_sm
  // blocks on an SM.
  std::vector<int> by_rows(nd);
  for (int d = 0; d < nd; ++d) by_rows[d] = d;
  std::stable_sort(by_rows.begin(), by_rows.end(),
                   [&](int a, int b) { return dims_params.dims[a].rows < dims_params.dims[b].rows; });
  // The direct form (sb_fact_direct_kernel) when every foreign key and
  // dimension key is int32 and the foreign-key columns are 16-byte aligned;
  // else the copy pipeline (sb_fact_kernel).
  direct = spec.direct && aligned;
  for (int d = 0; d < nd; ++d) direct = direct && fk_width[d] == 4 && dims_params.dims[d].key32;
  const int64_t masks_off = direct ? 0 : kSBBarBytes + spec.stages * stage_bytes;
  fact_params.masks_off = static_cast<int32_t>(masks_off);
  // Query masks are 32 bits wide for batches of at most 32 queries.
  mask_bytes = nq <= 32 ? 4 : 8;
  const int64_t rings_bytes = static_cast<int64_t>(direct ? kSBDirectWarps : kSBConsumerWarps) *
                              (mask_bytes == 4 ? sizeof(SBRings<uint32_t>) : sizeof(SBRings<uint64_t>));
  const int64_t block_target = std::min<int64_t>(kSBSmemBudget / std::max(1, spec.blocks_per_sm), kSBSmemPerBlockMax);
  const int64_t budget = std::max<int64_t>(0, block_target - masks_off - rings_bytes);
  int64_t staged = 0;  // bytes
  int n_staged = 0;
  for (int d = 0; d < nd; ++d) dims_params.dims[d].smem_off = -1;
  for (int d : by_rows) {
    SBDimDev& D = dims_params.dims[d];
    if (direct && n_staged == kSBFastStaged) break;
    const int64_t keys = (D.rows + 15) / 16 * 16;  // a dense key range needs one entry per row
    // the class -> mask table, each group column's values, one class byte per key
    const int64_t bytes = 256 * mask_bytes + keys * (1 + 4 * D.n_group);
    if (D.rows == 0 || staged + bytes > budget) continue;
    D.smem_off = static_cast<int32_t>(staged);
    D.smem_cap = static_cast<int32_t>(keys);
    staged += bytes;
    ++n_staged;
  }
  const int64_t rings_off = (masks_off + staged + 15) / 16 * 16;
  fact_params.rings_off = static_cast<int32_t>(rings_off);
  fact_smem = static_cast<size_t>(rings_off + rings_bytes);
  if (fact_smem > static_cast<size_t>(kSBSmemMaxDynamic))
    fail(GFPDB_EUNSUPPORTED, "itemsPerThread needs more shared memory than a block can have for these key widths");
  // Probe order: as given (a permutation of the dimensions), else the staged
  // dimensions, then the rest, each by row count.
  std::vector<int> order;
  if (!spec.probe_order.empty()) {
    std::vector<int> seen(nd, 0);
    if (static_cast<int>(spec.probe_order.size()) != nd) fail(GFPDB_EINVAL, "probeOrder must list every dimension once");
    for (int d : spec.probe_order) {
      if (d < 0 || d >= nd || seen[d]++) fail(GFPDB_EINVAL, "probeOrder must list every dimension once");
      order.push_back(d);
    }
  } else {
    for (int d : by_rows)
      if (dims_params.dims[d].smem_off >= 0) order.push_back(d);
    for (int d : by_rows)
      if (dims_params.dims[d].smem_off < 0) order.push_back(d);
  }
  for (int d = 0; d < nd; ++d) {
    fact_params.fd.fk_col[d] = fk_slot[d];
    fact_params.fd.order[d] = order[d];
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
  dq_buf = make_buffer(table_words * 8, s);
  drow_buf = make_buffer(table_words * 4, s);
  int64_t group_words = 0;
  for (int d = 0; d < nd; ++d) group_words += static_cast<int64_t>(dims_params.dims[d].mask + 1) * dims_params.dims[d].n_group;
  dg_buf = make_buffer(std::max<int64_t>(group_words, 1) * 4, s);
  dclass_buf = make_buffer(table_words, s);
  krange_buf = make_buffer(2 * kSBMaxDims * 8, s);
  masks_buf = make_buffer(std::max<int64_t>(mask_words, 1) * 8, s);
  gkeys_buf = make_buffer(static_cast<int64_t>(gcap) * 8, s);
  touched_buf = make_buffer(static_cast<int64_t>(gcap + 1) * 8, s);
  gaccs_buf = make_buffer(gslots * 8 * na, s);
  // status block, output count, then per-query counts, cursors and offsets
  misc_buf = make_buffer(sizeof(DevStatus) + 64 + 8 * (3 * kSBMaxQueries + 1) + 16, s);
  meta_buf = make_buffer(static_cast<int64_t>(hcols.size() * sizeof(DevCol) + hbase.size() * 8 + hrows.size() * 8 +
                                              kSBMaxDims * sizeof(SBSegments)),
                         s);
  out_cap = gslots;
  out_q = make_buffer(out_cap * 4, s);
  for (size_t g = 0; g < spec.group.size(); ++g) out_g[g] = make_buffer(out_cap * 4, s);
  for (int a = 0; a < na; ++a) out_a[a] = make_buffer(out_cap * 8, s);
  // wire pointers
  int64_t toff = 0, moff = 0, goff = 0;
  for (int d = 0; d < nd; ++d) {
    SBDimDev& D = dims_params.dims[d];
    D.slots = tables_buf->as<uint64_t>() + toff;
    D.qmask = masks_buf->as<uint64_t>() + moff;
    D.dq = dq_buf->as<uint64_t>() + toff;
    D.drow = drow_buf->as<uint32_t>() + toff;
    D.dclass = dclass_buf->as<uint8_t>() + toff;
    for (int c = 0; c < D.n_group; ++c) {
      D.dg[c] = dg_buf->as<int32_t>() + goff;
      goff += static_cast<int64_t>(D.mask + 1);
    }
    D.kmin_u = krange_buf->as<unsigned long long>() + d;
    D.kmax_u = krange_buf->as<unsigned long long>() + kSBMaxDims + d;
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
  SBSegments* dsegs = reinterpret_cast<SBSegments*>(drows + hrows.size());
  dims_params.segs = dsegs;
  // Host-resident fact columns that the direct fact pass reads only for
  // some rows (the foreign keys of dimensions it does not stage, and the
  // measures) are read in place from page-locked host memory; the columns
  // it reads in full are copied by every run (plan_host_copies).
  in_place.assign(nc, 0);
  n_in_place_fk = n_in_place_measures = 0;
  if (direct && !host_cols.empty()) {
    for (int c = 0; c < nc; ++c) {
      bool fk = false, staged_fk = false;
      for (int d = 0; d < nd; ++d)
        if (fk_slot[d] == c) {
          fk = true;
          staged_fk |= dims_params.dims[d].smem_off >= 0;
        }
      if (staged_fk) continue;
      std::vector<const void*> views(parts.size(), nullptr);
      bool ok = true;
      for (size_t pi = 0; pi < parts.size() && ok; ++pi) {
        const auto& col = parts[pi]->column(fact_cols[c]);
        const StarBatchHostColumn* h = nullptr;
        for (const auto& hc : host_cols)
          if (hc.dst == col->data) h = &hc;
        views[pi] = h != nullptr ? device_view_of_host(h->src) : nullptr;
        ok = views[pi] != nullptr;
      }
      if (!ok) continue;
      for (size_t pi = 0; pi < parts.size(); ++pi) hcols[pi * nc + c].data = views[pi];
      in_place[c] = 1;
      if (fk)
        ++n_in_place_fk;
      else
        ++n_in_place_measures;
    }
  }
  // Metadata goes up once, from host memory that this object keeps (so a
  // captured graph never needs it again).
  host_meta.assign(meta_buf->size(), 0);
  std::memcpy(host_meta.data(), hcols.data(), hcols.size() * sizeof(DevCol));
  std::memcpy(host_meta.data() + hcols.size() * sizeof(DevCol), hbase.data(), hbase.size() * 8);
  std::memcpy(host_meta.data() + hcols.size() * sizeof(DevCol) + hbase.size() * 8, hrows.data(), hrows.size() * 8);
  ranges_host_off = hcols.size() * sizeof(DevCol) + hbase.size() * 8 + hrows.size() * 8;
  fill_segments(spec.queries, nd, reinterpret_cast<SBSegments*>(host_meta.data() + ranges_host_off));
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
  fact_params.gkeys = gkeys_buf->as<uint64_t>();
  fact_params.gaccs = gaccs_buf->as<unsigned long long>();
  fact_params.gmask = gcap - 1;
  fact_params.touched = touched_buf->as<unsigned long long>();
  fact_params.st = st;
  fact_params.segs = dsegs;
  for (int d = 0; d < nd; ++d) fact_params.dims[d] = dims_params.dims[d];
  counter = reinterpret_cast<unsigned long long*>(misc + sizeof(DevStatus));
  qcount = reinterpret_cast<unsigned long long*>(misc + sizeof(DevStatus) + 64);
  qcursor = qcount + kSBMaxQueries;
  qoff = qcursor + kSBMaxQueries;
  gathered = qoff + kSBMaxQueries + 1;
  fact_params.gathered = gathered;
  fact_params.tile_begin = 0;
  fact_params.tile_end = n_tiles;
  plan_host_copies();
}

// Launches with at most as many blocks as are resident at once: tiles are
// striped over the grid, so a block that had to wait for a free SM would
// finish its stripe after everyone else.
template <int ITEMS, typename M>
static void launch_fact_items(const SBFactParams& p, size_t smem, int grid, cudaStream_t s) {
  // Opt in once to the largest dynamic size this engine asks for (static
  // plus dynamic shared memory above 48 KB needs it).
  static std::once_flag configured;
  std::call_once(configured, [] {
    GF_CUDA(cudaFuncSetAttribute(sb_fact_kernel<ITEMS, M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kSBSmemMaxDynamic)));
  });
  int per_sm = 0;
  GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sb_fact_kernel<ITEMS, M>, kSBFactThreads, smem));
  if (per_sm < 1) fail(GFPDB_EUNSUPPORTED, "the batched fact stage does not fit on an SM with these settings");
  const int resident = per_sm * num_sms();
  sb_fact_kernel<ITEMS, M><<<grid < resident ? grid : resident, kSBFactThreads, smem, s>>>(p);
}

template <typename M>
static void launch_fact_mask(const SBFactParams& p, size_t smem, int grid, cudaStream_t s) {
  switch (p.items) {
    case 1: launch_fact_items<1, M>(p, smem, grid, s); break;
    case 2: launch_fact_items<2, M>(p, smem, grid, s); break;
    case 4: launch_fact_items<4, M>(p, smem, grid, s); break;
    default: launch_fact_items<8, M>(p, smem, grid, s); break;
  }
}

template <int ITEMS, typename M>
static void launch_direct_items(const SBFactParams& p, size_t smem, int64_t tiles, cudaStream_t s) {
  static std::once_flag configured;
  std::call_once(configured, [] {
    GF_CUDA(cudaFuncSetAttribute(sb_fact_direct_kernel<ITEMS, M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kSBSmemMaxDynamic)));
  });
  int per_sm = 0;
  GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sb_fact_direct_kernel<ITEMS, M>, kSBDirectThreads,
                                                        smem));
  if (per_sm < 1) fail(GFPDB_EUNSUPPORTED, "the batched fact stage does not fit on an SM with these settings");
  int64_t grid = static_cast<int64_t>(per_sm) * num_sms();
  const int64_t need = (tiles + kSBDirectWarps - 1) / kSBDirectWarps;
  if (grid > need) grid = need;
  sb_fact_direct_kernel<ITEMS, M><<<static_cast<int>(grid), kSBDirectThreads, smem, s>>>(p);
}

template <typename M>
static void launch_direct_mask(const SBFactParams& p, size_t smem, int64_t tiles, cudaStream_t s) {
  switch (p.items) {
    case 1: launch_direct_items<1, M>(p, smem, tiles, s); break;
    case 2: launch_direct_items<2, M>(p, smem, tiles, s); break;
    case 4: launch_direct_items<4, M>(p, smem, tiles, s); break;
    default: launch_direct_items<8, M>(p, smem, tiles, s); break;
  }
}

void StarBatchState::launch_fact(int grid, cudaStream_t s) {
  if (direct) {
    const int64_t tiles = fact_params.tile_end - fact_params.tile_begin;
    if (mask_bytes == 4)
      launch_direct_mask<uint32_t>(fact_params, fact_smem, tiles, s);
    else
      launch_direct_mask<uint64_t>(fact_params, fact_smem, tiles, s);
    return;
  }
  if (mask_bytes == 4)
    launch_fact_mask<uint32_t>(fact_params, fact_smem, grid, s);
  else
    launch_fact_mask<uint64_t>(fact_params, fact_smem, grid, s);
}

// The fact pass over tiles [begin, end), which hold `rows` fact rows.
static void fact_pass(StarBatchState& b, int64_t begin, int64_t end, int64_t rows, cudaStream_t s) {
  if (end <= begin) return;
  int64_t grid = static_cast<int64_t>(num_sms()) * b.spec.blocks_per_sm;
  if (grid > end - begin) grid = end - begin;
  b.fact_params.tile_begin = begin;
  b.fact_params.tile_end = end;
  const char* name = b.direct ? "sb_fact_direct_kernel" : "sb_fact_kernel";
  ProfScope prof(name, s);
  b.launch_fact(static_cast<int>(grid), s);
  after_launch(name);
  // algorithmic bytes: every foreign key of every fact row of these tiles
  // read once (the measures of the few surviving rows are not counted)
  double fk_bytes = 0;
  for (int d = 0; d < b.fact_params.n_dims; ++d) fk_bytes += b.fact_params.fk_width[d];
  prof.stop(static_cast<double>(rows) * fk_bytes);
}

void StarBatchState::run(cudaStream_t s) {
  const bool host = !dim_copies.empty() || !group_copies.empty();
  if (host) {
    // host-resident inputs: copies on their own stream, forked from s (the
    // caller counts host_bytes per run: a captured run copies too)
    GF_CUDA(cudaEventRecord(events[0], s));
    GF_CUDA(cudaStreamWaitEvent(copy_stream, events[0], 0));
    for (const Copy& c : dim_copies)
      GF_CUDA(cudaMemcpyAsync(c.dst, c.src, static_cast<size_t>(c.bytes), cudaMemcpyHostToDevice, copy_stream));
    GF_CUDA(cudaEventRecord(events[1], copy_stream));
    for (size_t g = 0; g < group_copies.size(); ++g) {
      for (const Copy& c : group_copies[g])
        GF_CUDA(cudaMemcpyAsync(c.dst, c.src, static_cast<size_t>(c.bytes), cudaMemcpyHostToDevice, copy_stream));
      GF_CUDA(cudaEventRecord(events[2 + g], copy_stream));
    }
  }
  // clear: join tables to empty, group keys to empty, accumulators / status / counters to zero
  GF_CUDA(cudaMemsetAsync(tables_buf->data(), 0xFF, tables_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(dq_buf->data(), 0, dq_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(drow_buf->data(), 0xFF, drow_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(dclass_buf->data(), kSBNoRow, dclass_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(krange_buf->data(), 0xFF, kSBMaxDims * 8, s));  // minima
  GF_CUDA(cudaMemsetAsync(krange_buf->as<char>() + kSBMaxDims * 8, 0, kSBMaxDims * 8, s));  // maxima
  GF_CUDA(cudaMemsetAsync(gkeys_buf->data(), 0xFF, gkeys_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(touched_buf->data(), 0, touched_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(gaccs_buf->data(), 0, gaccs_buf->size(), s));
  GF_CUDA(cudaMemsetAsync(misc_buf->data(), 0, misc_buf->size(), s));
  const int sms = num_sms();
  if (host) GF_CUDA(cudaStreamWaitEvent(s, events[1], 0));  // the dimensions have landed
  {
    int64_t max_rows = 1;
    for (int d = 0; d < dims_params.n_dims; ++d) max_rows = std::max<int64_t>(max_rows, dims_params.dims[d].rows);
    int64_t bx = (max_rows + kSBThreads - 1) / kSBThreads;
    if (bx > 64) bx = 64;
    ProfScope prof("sb_range_kernel", s);
    sb_range_kernel<<<dim3(static_cast<unsigned>(bx), static_cast<unsigned>(dims_params.n_dims)), kSBThreads, 0, s>>>(
        dims_params);
    after_launch("sb_range_kernel");
    prof.stop(static_cast<double>(dims_params.total_rows) * 4.0);
  }
  {
    int64_t blocks = (dims_params.total_rows + kSBThreads - 1) / kSBThreads;
    if (blocks > sms * 8) blocks = sms * 8;
    if (blocks < 1) blocks = 1;
    ProfScope prof("sb_dims_kernel", s);
    sb_dims_kernel<<<static_cast<int>(blocks), kSBThreads, 0, s>>>(dims_params);
    after_launch("sb_dims_kernel");
    prof.stop(static_cast<double>(dims_params.total_rows) * 12.0);
  }
  if (host) {
    for (size_t g = 0; g < group_tiles.size(); ++g) {
      GF_CUDA(cudaStreamWaitEvent(s, events[2 + g], 0));
      fact_pass(*this, group_tiles[g].begin, group_tiles[g].end, group_tiles[g].rows, s);
    }
  } else {
    fact_pass(*this, 0, n_tiles, fact_rows, s);
  }
  {
    SBFinalParams fp;
    std::memset(&fp, 0, sizeof(fp));
    fp.gkeys = gkeys_buf->as<uint64_t>();
    fp.touched = touched_buf->as<unsigned long long>();
    fp.gaccs = gaccs_buf->as<unsigned long long>();
    fp.slots = gcap + 1;
    fp.n_queries = static_cast<int32_t>(spec.queries.size());
    fp.n_aggs = static_cast<int32_t>(spec.aggs.size());
    fp.n_group = static_cast<int32_t>(spec.group.size());
    fp.out_q = out_q->as<int32_t>();
    for (size_t g = 0; g < spec.group.size(); ++g) fp.out_g[g] = out_g[g]->data();
    for (size_t a = 0; a < spec.aggs.size(); ++a) fp.out_a[a] = out_a[a]->as<long long>();
    fp.counter = counter;
    fp.qcount = qcount;
    fp.qcursor = qcursor;
    fp.qoff = qoff;
    const uint64_t total = fp.slots * static_cast<uint64_t>(fp.n_queries);
    int64_t cblocks = static_cast<int64_t>((fp.slots + 255) / 256);
    if (cblocks > sms * 2) cblocks = sms * 2;
    sb_count_kernel<<<static_cast<int>(cblocks), 256, 0, s>>>(fp);
    after_launch("sb_count_kernel");
    int64_t blocks = static_cast<int64_t>((total + 255) / 256);
    if (blocks > sms * 8) blocks = sms * 8;
    ProfScope prof("sb_final_kernel", s);
    sb_final_kernel<<<static_cast<int>(blocks), 256, 0, s>>>(fp);
    after_launch("sb_final_kernel");
    prof.stop(static_cast<double>(total) * 8.0 * (1 + fp.n_aggs));
  }
}

void StarBatchState::set_ranges(const std::vector<std::vector<std::pair<int64_t, int64_t>>>& q, cudaStream_t s) {
  const int nq = static_cast<int>(spec.queries.size());
  const int nd = static_cast<int>(spec.dims.size());
  if (static_cast<int>(q.size()) > nq) fail(GFPDB_EINVAL, "more queries than the batch was prepared for");
  std::vector<std::vector<std::pair<int64_t, int64_t>>> all(nq);
  for (int i = 0; i < nq; ++i) {
    const bool used = i < static_cast<int>(q.size());
    if (used && static_cast<int>(q[i].size()) != nd) fail(GFPDB_EINVAL, "each query needs one range per dimension");
    // an unused slot: the empty range [1, 0] on every dimension
    all[i] = used ? q[i] : std::vector<std::pair<int64_t, int64_t>>(nd, std::make_pair(int64_t{1}, int64_t{0}));
  }
  fill_segments(all, nd, reinterpret_cast<SBSegments*>(host_meta.data() + ranges_host_off));
  GF_CUDA(cudaMemcpyAsync(meta_buf->as<char>() + ranges_host_off, host_meta.data() + ranges_host_off,
                          static_cast<size_t>(nd) * sizeof(SBSegments), cudaMemcpyHostToDevice, s));
  sync(s);  // host_meta may be rewritten by the next call
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
