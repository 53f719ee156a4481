// Fused selection: predicate (CNF leaf program) + bloom probes + stable
// compaction + projection in one pass.
//
// Replaces, as one kernel, what the reference runs as separate passes per
// 100k-row batch: Gandiva's selection vector (Filter::computeSelectionVector),
// the pass-through projector gather (Filter::evaluateBySelectionVector,
// fpdb-expression-gandiva/src/Filter.cpp:178-225), and the bloom hash / find /
// arrow::compute::Filter chain (BloomFilterUseKernel::filterRecordBatch,
// fpdb-executor/src/physical/bloomfilter/BloomFilterUseKernel.cpp:180-207).
//
// Work decomposition: persistent CTAs of 256 threads take 2048-row tiles in
// increasing order from an atomic ticket; each thread owns 8 consecutive rows
// (one 32-byte sector of an int32 column, read with two 128-bit loads). Leaves
// and probes are evaluated in order and a later column is only loaded for the
// rows still alive, so a selective early term saves the DRAM sectors of later
// columns. Selected rows are ranked with a block scan plus decoupled
// look-back, giving stable (input-order) output in a single pass; each thread
// then moves its own selected rows of every projected column with 128-bit
// loads, so a sparse tile only touches the sectors holding selected rows.
// Small bloom filters are staged in shared memory once per CTA. Inputs whose
// row count lives on the device (deferred sizes) are read with that count.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <type_traits>

#include "../host/handles.h"
#include "bloom.cuh"
#include "eval.cuh"
#include "launch.h"

namespace gfpdb {

namespace {

constexpr int kSelThreads = 256;
constexpr int kSelItems = 8;
constexpr int kSelTile = kSelThreads * kSelItems;
constexpr int kBloomSmemBudget = 96 * 1024;

struct BloomDev {
  const uint32_t* blocks;
  const uint64_t* nblocks_dev;  // set when the filter's size lives on the device
  const int32_t* valid_dev;
  uint32_t num_blocks;
  int16_t col;
  int8_t num_hashes;
  int8_t valid;
  int32_t smem_word;      // < 0: probe from global memory
  int32_t smem_cap_words; // shared-memory words reserved for this filter
};

struct OutCol {
  const void* src;
  void* dst;
  int32_t width;
  int32_t aligned;  // src is 16-byte aligned: 128-bit loads allowed
};

struct SelectParams {
  int64_t n_rows;            // exact row count, or the capacity when n_dev is set
  const int64_t* n_dev;      // device row count of a deferred input
  int64_t n_tiles;
  int32_t n_cols;
  int32_t n_probes;
  int32_t n_out;
  int32_t smem_words;
  int32_t aligned;
  int32_t pad;
  DevCol cols[kMaxCols];
  BloomDev probes[kMaxBlooms];
  OutCol outs[kMaxCols];
  int32_t* out_rowids;
  uint64_t* tile_status;
  uint32_t* ticket;
  DevStatus* status;
  Program prog;
};

__device__ __forceinline__ void load8(const DevCol& c, int64_t row0, uint32_t need, bool vec, int64_t v[8]) {
  if (c.type == CT_I64 || c.type == CT_F64) {
    const long long* p = static_cast<const long long*>(c.data) + row0;
    if (vec) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if ((need >> (4 * h)) & 0xFu) {
          const longlong2 a = __ldg(reinterpret_cast<const longlong2*>(p) + 2 * h);
          const longlong2 b = __ldg(reinterpret_cast<const longlong2*>(p) + 2 * h + 1);
          v[4 * h + 0] = a.x;
          v[4 * h + 1] = a.y;
          v[4 * h + 2] = b.x;
          v[4 * h + 3] = b.y;
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kSelItems; ++k)
        if ((need >> k) & 1u) v[k] = __ldg(p + k);
    }
  } else {
    const int* p = static_cast<const int*>(c.data) + row0;
    if (vec) {
      const int4 a = __ldg(reinterpret_cast<const int4*>(p));
      const int4 b = __ldg(reinterpret_cast<const int4*>(p) + 1);
      v[0] = a.x;
      v[1] = a.y;
      v[2] = a.z;
      v[3] = a.w;
      v[4] = b.x;
      v[5] = b.y;
      v[6] = b.z;
      v[7] = b.w;
    } else {
#pragma unroll
      for (int k = 0; k < kSelItems; ++k)
        if ((need >> k) & 1u) v[k] = __ldg(p + k);
    }
  }
}

__device__ __forceinline__ void operand8(const SelectParams& p, const Operand& o, int64_t row0, uint32_t need,
                                         bool vec, int64_t v[8]) {
  if (o.kind == OPND_COL) {
    load8(p.cols[o.col], row0, need, vec, v);
  } else if (o.kind == OPND_LIT) {
#pragma unroll
    for (int k = 0; k < kSelItems; ++k) v[k] = o.lit.i;
  } else {
#pragma unroll
    for (int k = 0; k < kSelItems; ++k)
      if ((need >> k) & 1u) v[k] = eval_prog(p.prog, p.cols, o.prog_begin, o.prog_len, row0 + k, p.status);
  }
}

template <typename T>
__device__ __forceinline__ uint32_t compare8(int op, const int64_t a[8], const int64_t b[8]) {
  uint32_t r = 0;
  auto val = [](int64_t x) -> T {
    if constexpr (std::is_floating_point_v<T>) {
      return __longlong_as_double(x);
    } else {
      return static_cast<T>(x);
    }
  };
  switch (op) {
    case LO_LT:
#pragma unroll
      for (int k = 0; k < 8; ++k) r |= static_cast<uint32_t>(val(a[k]) < val(b[k])) << k;
      break;
    case LO_LE:
#pragma unroll
      for (int k = 0; k < 8; ++k) r |= static_cast<uint32_t>(val(a[k]) <= val(b[k])) << k;
      break;
    case LO_GT:
#pragma unroll
      for (int k = 0; k < 8; ++k) r |= static_cast<uint32_t>(val(a[k]) > val(b[k])) << k;
      break;
    case LO_GE:
#pragma unroll
      for (int k = 0; k < 8; ++k) r |= static_cast<uint32_t>(val(a[k]) >= val(b[k])) << k;
      break;
    case LO_EQ:
#pragma unroll
      for (int k = 0; k < 8; ++k) r |= static_cast<uint32_t>(val(a[k]) == val(b[k])) << k;
      break;
    default:
#pragma unroll
      for (int k = 0; k < 8; ++k) r |= static_cast<uint32_t>(val(a[k]) != val(b[k])) << k;
      break;
  }
  return r;
}

__device__ __forceinline__ uint32_t leaf8(const SelectParams& p, const Leaf& L, int64_t row0, uint32_t need,
                                          bool vec) {
  if (need == 0) return 0;
  if (L.op == LO_TRUE) return need;
  if (L.op == LO_FALSE) return 0;
  if (L.op == LO_STR_EQ || L.op == LO_STR_NE || L.op == LO_LIKE || L.op == LO_NOT_LIKE) {
    const DevCol& c = p.cols[L.lhs.col];
    uint32_t r = 0;
    for (int k = 0; k < kSelItems; ++k) {
      if (!((need >> k) & 1u)) continue;
      if (string_test(L.op, c, row0 + k, p.prog.strpool + L.str_begin, L.str_len, L.rhs.col == 1, L.rhs.prog_begin,
                      L.rhs.prog_len))
        r |= 1u << k;
    }
    return r;
  }
  if (L.op == LO_STRCOL_EQ || L.op == LO_STRCOL_NE) {
    const DevCol& c1 = p.cols[L.lhs.col];
    const DevCol& c2 = p.cols[L.rhs.col];
    const uint8_t* s1 = static_cast<const uint8_t*>(c1.data);
    const uint8_t* s2 = static_cast<const uint8_t*>(c2.data);
    uint32_t r = 0;
    for (int k = 0; k < kSelItems; ++k) {
      if (!((need >> k) & 1u)) continue;
      const int32_t b1 = c1.offsets[row0 + k], e1 = c1.offsets[row0 + k + 1];
      const int32_t b2 = c2.offsets[row0 + k], e2 = c2.offsets[row0 + k + 1];
      bool eq = (e1 - b1) == (e2 - b2);
      for (int32_t i = 0; eq && i < e1 - b1; ++i) eq = s1[b1 + i] == s2[b2 + i];
      if (eq == (L.op == LO_STRCOL_EQ)) r |= 1u << k;
    }
    return r;
  }
  int64_t a[8], b[8];
  operand8(p, L.lhs, row0, need, vec, a);
  operand8(p, L.rhs, row0, need, vec, b);
  const uint32_t r = L.cmp_vt == VT_F64 ? compare8<double>(L.op, a, b) : compare8<int64_t>(L.op, a, b);
  return r & need;
}

// kPred = false compiles the probe-only form (BloomFilterUse chains), which
// needs far fewer registers than the general CNF evaluator.
template <bool kPred>
__global__ void __launch_bounds__(kSelThreads) select_kernel(const __grid_constant__ SelectParams p) {
  extern __shared__ __align__(16) uint32_t s_bloom[];
  __shared__ int s_warp[kSelThreads / 32 + 1];
  __shared__ uint32_t s_tile;
  __shared__ uint64_t s_base;
  __shared__ uint32_t s_nblocks[kMaxBlooms];

  // Row count: exact, or produced on the device by the previous operator.
  const int64_t n_rows = clamp_rows(p.n_dev, p.n_rows);
  const int64_t n_tiles = (n_rows + kSelTile - 1) / kSelTile;

  // Filter sizes may also live on the device (filters built from deferred
  // inputs). Stage each filter in shared memory when it fits its slot.
  uint32_t staged = 0, valid = 0;
#pragma unroll 1
  for (int pi = 0; pi < p.n_probes; ++pi) {
    const BloomDev& b = p.probes[pi];
    const uint32_t nb = b.nblocks_dev ? static_cast<uint32_t>(*b.nblocks_dev) : b.num_blocks;
    if (threadIdx.x == 0) s_nblocks[pi] = nb;
    const bool v = b.valid_dev ? (*b.valid_dev != 0) : (b.valid != 0);
    if (v) valid |= 1u << pi;
    if (v && b.smem_word >= 0 && nb * 8 <= static_cast<uint32_t>(b.smem_cap_words)) {
      staged |= 1u << pi;
      const uint4* src = reinterpret_cast<const uint4*>(b.blocks);
      uint4* dst = reinterpret_cast<uint4*>(s_bloom + b.smem_word);
      for (uint32_t i = threadIdx.x; i < nb * 2; i += kSelThreads) dst[i] = __ldg(src + i);
    }
  }
  __syncthreads();

  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(p.ticket, 1u);
    __syncthreads();
    const int64_t tile = s_tile;
    if (tile >= n_tiles) break;
    const int64_t row0 = tile * kSelTile + static_cast<int64_t>(threadIdx.x) * kSelItems;
    const bool full = row0 + kSelItems <= n_rows;
    const bool vec = full && p.aligned;
    uint32_t mask;
    if (full) {
      mask = 0xFFu;
    } else {
      const int64_t rem = n_rows - row0;
      mask = rem <= 0 ? 0u : ((1u << rem) - 1u);
    }

    // Bloom probes (the predicate-transfer chain), most selective first as
    // the caller ordered them.
#pragma unroll 1
    for (int pi = 0; pi < p.n_probes; ++pi) {
      if (!((valid >> pi) & 1u) || mask == 0) continue;
      const BloomDev& b = p.probes[pi];
      const uint32_t nb = s_nblocks[pi];
      int64_t keys[8];
      load8(p.cols[b.col], row0, mask, vec, keys);
      uint32_t keep = 0;
      const bool in_smem = (staged >> pi) & 1u;
#pragma unroll
      for (int k = 0; k < kSelItems; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const uint64_t h = bloom_hash(keys[k]);
        const uint32_t blk = bloom_block_of(h, nb);
        bool ok;
        if (in_smem) {
          ok = bloom_test(s_bloom + b.smem_word + blk * 8, h, b.num_hashes);
        } else {
          const uint4* words = reinterpret_cast<const uint4*>(b.blocks + static_cast<uint64_t>(blk) * 8);
          uint32_t w[8];
          const uint4 lo = __ldg(words);
          const uint4 hi = __ldg(words + 1);
          w[0] = lo.x; w[1] = lo.y; w[2] = lo.z; w[3] = lo.w;
          w[4] = hi.x; w[5] = hi.y; w[6] = hi.z; w[7] = hi.w;
          ok = bloom_test(w, h, b.num_hashes);
        }
        keep |= static_cast<uint32_t>(ok) << k;
      }
      mask &= keep;
    }

    // Predicate in CNF.
    if constexpr (kPred) {
      for (int c = 0; c < p.prog.n_clauses; ++c) {
        if (mask == 0) break;
        uint32_t cm = 0;
        for (int l = p.prog.clause_begin[c]; l < p.prog.clause_begin[c + 1]; ++l)
          cm |= leaf8(p, p.prog.leaves[l], row0, mask & ~cm, vec);
        mask &= cm;
      }
    }

    // Rank the selected rows: block scan + decoupled look-back.
    const int cnt = __popc(mask);
    int tile_total;
    const int excl = block_exclusive_sum<kSelThreads>(cnt, &tile_total, s_warp);
    if (threadIdx.x < 32) {
      const uint64_t b = lookback_exclusive(p.tile_status, tile, static_cast<uint64_t>(tile_total), p.status);
      if (threadIdx.x == 0) s_base = b;
    }
    __syncthreads();
    const int64_t base = static_cast<int64_t>(s_base);
    // Projection: each thread moves its own selected rows. A thread with any
    // selected row loads its 8 rows of a column with 128-bit loads (the
    // sectors a row-granular gather would touch anyway) and writes the
    // selected values to consecutive output slots; threads with none load
    // nothing, so sparse tiles skip most sectors of unselected columns.
    if (mask != 0) {
      const int64_t out0 = base + excl;
#pragma unroll 1
      for (int j = 0; j < p.n_out; ++j) {
        const OutCol& oc = p.outs[j];
        int64_t v[8];
        const DevCol c{oc.src, nullptr, oc.width == 8 ? CT_I64 : CT_I32, 0};
        load8(c, row0, mask, vec && oc.aligned, v);
        int o = 0;
        if (oc.width == 8) {
          long long* dst = static_cast<long long*>(oc.dst) + out0;
#pragma unroll
          for (int k = 0; k < kSelItems; ++k)
            if ((mask >> k) & 1u) dst[o++] = v[k];
        } else {
          int* dst = static_cast<int*>(oc.dst) + out0;
#pragma unroll
          for (int k = 0; k < kSelItems; ++k)
            if ((mask >> k) & 1u) dst[o++] = static_cast<int>(v[k]);
        }
      }
      if (p.out_rowids != nullptr) {
        int o = 0;
#pragma unroll
        for (int k = 0; k < kSelItems; ++k)
          if ((mask >> k) & 1u) p.out_rowids[out0 + o++] = static_cast<int32_t>(row0 + k);
      }
    }
    if (tile == n_tiles - 1 && threadIdx.x == 0) p.status->value = base + tile_total;
    __syncthreads();
  }
}

// Resident CTAs per SM for a variant and dynamic shared-memory size, cached
// (the occupancy query is not free and the answer never changes).
int select_blocks_per_sm(bool with_pred, size_t dyn) {
  static std::mutex mu;
  static std::map<std::pair<bool, size_t>, int> cache;
  static bool attr_set[2] = {false, false};
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(with_pred, dyn);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  const void* fn = with_pred ? reinterpret_cast<const void*>(select_kernel<true>)
                             : reinterpret_cast<const void*>(select_kernel<false>);
  if (!attr_set[with_pred]) {
    GF_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kBloomSmemBudget));
    attr_set[with_pred] = true;
  }
  int per_sm = 0;
  GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSelThreads, dyn));
  if (per_sm < 1) per_sm = 1;
  cache[key] = per_sm;
  return per_sm;
}

// A predicate leaf of the simple form: an integer column against an integer
// literal, the comparison reduced to a 4-bit truth table over
// (value < literal, value == literal). The compact and the two-pass
// selections evaluate a CNF of such leaves.
constexpr int kSimpleMaxLeaves = 8;

struct SimpleLeaf {
  const void* col;
  int64_t lit;
  int8_t wide;          // 1: int64 column; 0: int32 / date32
  int8_t truth;         // bit (2 * (v < lit) + (v == lit)) set when the leaf holds
  int8_t clause_start;  // 1: first leaf of its clause
  int8_t pad[5];
};

// The predicate of p as simple leaves in clause order, or false when a leaf
// has another form, a clause is empty, there are more than max leaves, or a
// leaf's column is not 16-byte aligned.
bool simple_leaves(const SelectParams& p, SimpleLeaf* out, int max, int* n_out) {
  auto aligned = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  // truth tables over (lt, eq) for LO_LT, LO_LE, LO_GT, LO_GE, LO_EQ, LO_NE
  static const int8_t kTruth[6] = {4, 6, 1, 3, 2, 5};
  static const int8_t kMirror[6] = {LO_GT, LO_GE, LO_LT, LO_LE, LO_EQ, LO_NE};
  const Program& g = p.prog;
  int n = 0;
  for (int c = 0; c < g.n_clauses; ++c) {
    if (g.clause_begin[c] >= g.clause_begin[c + 1]) return false;
    for (int l = g.clause_begin[c]; l < g.clause_begin[c + 1]; ++l) {
      const Leaf& L = g.leaves[l];
      if (L.op < LO_LT || L.op > LO_NE || L.cmp_vt != VT_I64) return false;
      Operand a = L.lhs, b = L.rhs;
      int op = L.op;
      if (a.kind == OPND_LIT && b.kind == OPND_COL) {
        std::swap(a, b);
        op = kMirror[op];
      }
      if (a.kind != OPND_COL || b.kind != OPND_LIT || b.vt != VT_I64) return false;
      const DevCol& dc = p.cols[a.col];
      if ((dc.type != CT_I32 && dc.type != CT_I64 && dc.type != CT_DATE32) || !aligned(dc.data)) return false;
      if (n == max) return false;
      SimpleLeaf& o = out[n++];
      o = SimpleLeaf{};
      o.col = dc.data;
      o.lit = b.lit.i;
      o.wide = dc.type == CT_I64 ? 1 : 0;
      o.truth = kTruth[op];
      o.clause_start = l == g.clause_begin[c] ? 1 : 0;
    }
  }
  *n_out = n;
  return true;
}

// ---------------------------------------------------------------------------
// Probe-only selection over a large input (the BloomFilterUse chain over the
// fact table), in two passes.
// Pass 1 (select_probe_kernel): warps work on their own 256-row slices of the
// input (32 lanes x 8 rows), taken by a fixed stride, with no barrier
// between warps: a lane loads its 8 keys of the first probe with 16-byte
// loads, tests them against the first filter (staged in shared memory once
// per CTA), the warp compacts its survivors with a ballot scan into its own
// row list, tests the later probes over that list only (their keys read
// directly for the survivors, all of a row's keys in one memory round trip),
// and writes the slice's selected row ids, in order, into the slice's part of
// a row-id buffer, with the slice's count. A warp waiting on memory for its
// later probes holds up no other warp.
// Pass 2 (select_gather_kernel): each CTA sums the counts before its range of
// slices and moves each slice's selected rows of every projected column to
// their output offsets.
// Output order is input order, as in the single-pass kernel.
constexpr int kPwThreads = 256;                 // 8 warps
constexpr int kGatherSlices = kSelThreads;     // slices per range of the gather pass (one per thread)
constexpr int kPwRows = 32 * kSelItems;         // rows per warp slice
constexpr int64_t kSpMinRows = int64_t{1} << 20;  // below this select_kernel's tiles all start at once
constexpr int64_t kSpMaxDynamic = 96 * 1024;    // the staged filters in shared memory
static_assert(kBloomSmemBudget <= kSpMaxDynamic, "the filters' shared-memory layout fits a probe launch");

// The first probe over a thread's 8 rows: the bloom test of each key with NH
// hashes, bit positions from the low 32 bits of the key's hash (bloom.cuh).
// IN_SMEM: the filter sits in shared memory (the pointer derives from the
// kernel's shared array, so the tests compile to shared-memory loads); else
// it is read through L1/L2.
template <bool IN_SMEM, int NH>
__device__ __forceinline__ uint32_t probe8(const uint32_t* blocks, uint32_t nb, const int64_t keys[8], uint32_t mask) {
  uint32_t keep = 0;
#pragma unroll
  for (int kk = 0; kk < kSelItems; ++kk) {
    const uint64_t h = bloom_hash(keys[kk]);
    const uint32_t* blk = blocks + static_cast<uint64_t>(bloom_block_of(h, nb)) * 8;
    const uint32_t lo = static_cast<uint32_t>(h);
    uint32_t ok = 1u;
#pragma unroll
    for (int i = 0; i < NH; ++i) {
      const uint32_t b = (lo >> (8 * i)) & 0xFFu;
      const uint32_t w = IN_SMEM ? blk[b >> 5] : __ldg(blk + (b >> 5));
      ok &= w >> (b & 31);
    }
    keep |= (ok & 1u) << kk;
  }
  return keep & mask;
}

template <bool IN_SMEM>
__device__ __forceinline__ uint32_t probe8_first(const uint32_t* blocks, uint32_t nb, int num_hashes,
                                                 const int64_t keys[8], uint32_t mask) {
  switch (num_hashes) {
    case 1: return probe8<IN_SMEM, 1>(blocks, nb, keys, mask);
    case 2: return probe8<IN_SMEM, 2>(blocks, nb, keys, mask);
    case 3: return probe8<IN_SMEM, 3>(blocks, nb, keys, mask);
    default: return probe8<IN_SMEM, 4>(blocks, nb, keys, mask);
  }
}

// The predicate of a two-pass selection (simple leaves, AND of ORs).
struct StreamPred {
  int32_t n_leaves;
  int32_t pad;
  SimpleLeaf leaves[kSimpleMaxLeaves];
};

// kPred = false compiles the probe-only form, which needs fewer registers.
// kLater: the number of probes after the first (1 to 3, their loop unrolled
// exactly), 0 for none, -1 for more (a loop over up to kMaxBlooms - 1).
template <bool kPred, int kLater>
__global__ void __launch_bounds__(kPwThreads, kPred ? 4 : 5) select_probe_kernel(const __grid_constant__ SelectParams p,
                                                                  const __grid_constant__ StreamPred sp,
                                                                  int32_t* __restrict__ rowlist,
                                                                  unsigned int* __restrict__ range_totals) {
  extern __shared__ __align__(16) uint32_t s_filter[];  // the staged filters, at their smem_word
  __shared__ uint16_t s_list[kPwThreads / 32][kPwRows];  // per warp: its slice's survivors
  __shared__ uint32_t s_nblocks[kMaxBlooms];
  __shared__ const uint32_t* s_blocks[kMaxBlooms];  // each filter's blocks: shared memory when staged
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t n_rows = clamp_rows(p.n_dev, p.n_rows);
  const int64_t n_slices = (n_rows + kPwRows - 1) / kPwRows;

  uint32_t valid = 0;
  bool staged = false;
#pragma unroll 1
  for (int pi = 0; pi < p.n_probes; ++pi) {
    const BloomDev& b = p.probes[pi];
    const uint32_t nb = b.nblocks_dev ? static_cast<uint32_t>(*b.nblocks_dev) : b.num_blocks;
    if (threadIdx.x == 0) s_nblocks[pi] = nb;
    const bool v = b.valid_dev ? (*b.valid_dev != 0) : (b.valid != 0);
    if (v) valid |= 1u << pi;
    const bool stage = v && b.smem_word >= 0 && nb * 8 <= static_cast<uint32_t>(b.smem_cap_words);
    if (threadIdx.x == 0) s_blocks[pi] = stage ? s_filter + b.smem_word : b.blocks;
    if (stage) {
      if (pi == 0) staged = true;
      const uint4* src = reinterpret_cast<const uint4*>(b.blocks);
      uint4* dst = reinterpret_cast<uint4*>(s_filter + b.smem_word);
      for (uint32_t i = threadIdx.x; i < nb * 2; i += kPwThreads) dst[i] = __ldg(src + i);
    }
  }
  __syncthreads();  // the only block-wide barrier: warps are independent below

  const BloomDev& b0 = p.probes[0];
  const uint32_t nb0 = s_nblocks[0];
  const DevCol& kc0 = p.cols[b0.col];
  const bool vec0 = (reinterpret_cast<uintptr_t>(kc0.data) & 15u) == 0;
  uint16_t* list = s_list[warp];
  const uint32_t lane_lt = (1u << lane) - 1u;
  const int64_t n_warps = static_cast<int64_t>(gridDim.x) * (kPwThreads / 32);
  for (int64_t sl = static_cast<int64_t>(blockIdx.x) * (kPwThreads / 32) + warp; sl < n_slices; sl += n_warps) {
    const int64_t start = sl * kPwRows;
    const int r_in = lane * kSelItems;
    const int64_t row0 = start + r_in;
    const int64_t rem = n_rows - row0;
    const bool full = rem >= kSelItems;
    uint32_t mask = full ? 0xFFu : (rem <= 0 ? 0u : ((1u << rem) - 1u));
    // (0) the predicate over this lane's 8 rows (16-byte loads when full)
    if (kPred && mask != 0) {
      uint32_t all = mask, any = 0;
#pragma unroll 1
      for (int l = 0; l < sp.n_leaves; ++l) {
        const SimpleLeaf& L = sp.leaves[l];
        if (L.clause_start && l > 0) {
          all &= any;
          any = 0;
        }
        int64_t v[kSelItems];
        load8(DevCol{L.col, nullptr, L.wide ? CT_I64 : CT_I32, 0}, row0, mask, full, v);
#pragma unroll
        for (int kk = 0; kk < kSelItems; ++kk) {
          const uint32_t idx = (static_cast<uint32_t>(v[kk] < L.lit) << 1) | static_cast<uint32_t>(v[kk] == L.lit);
          any |= ((static_cast<uint32_t>(L.truth) >> idx) & 1u) << kk;
        }
      }
      mask = all & any;
    }
    // (1) the first probe over this lane's 8 rows
    if ((valid & 1u) && mask != 0) {
      int64_t keys[kSelItems];
      load8(kc0, row0, mask, full && vec0, keys);
      if (!full) {
#pragma unroll
        for (int kk = 0; kk < kSelItems; ++kk)
          if (!((mask >> kk) & 1u)) keys[kk] = 0;  // a defined key for the rows past the end (masked below)
      }
      mask &= staged ? probe8_first<true>(s_filter, nb0, b0.num_hashes, keys, mask)
                     : probe8_first<false>(b0.blocks, nb0, b0.num_hashes, keys, mask);
    }
    // (2) the survivors, in row order, into the warp's list
    int n_alive;
    {
      const int c = __popc(mask);
      int incl = c;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
      }
      n_alive = __shfl_sync(0xffffffffu, incl, 31);
      int o = incl - c;
#pragma unroll
      for (int kk = 0; kk < kSelItems; ++kk)
        if ((mask >> kk) & 1u) list[o++] = static_cast<uint16_t>(r_in + kk);
      __syncwarp();
    }
    // (3) the later probes over the list, compacted in place (order kept: a
    // compacted position never passes the position it was read from); each
    // survivor's later keys are loaded together, the filters tested from
    // shared memory where staged
    if (kLater != 0 && n_alive > 0) {
      constexpr int NL = kLater > 0 ? kLater : kMaxBlooms - 1;
      const int nl = kLater > 0 ? kLater : p.n_probes - 1;
      int m = 0;
      for (int base = 0; base < n_alive; base += 32) {
        const int idx = base + lane;
        bool alive = idx < n_alive;
        const int r = alive ? list[idx] : 0;
        int64_t later[NL];
#pragma unroll
        for (int j = 0; j < NL; ++j) {
          const int pi = j + 1;
          later[j] = (j < nl && alive && ((valid >> pi) & 1u)) ? load_int(p.cols[p.probes[pi].col], start + r) : 0;
        }
#pragma unroll
        for (int j = 0; j < NL; ++j) {
          const int pi = j + 1;
          if (j < nl && alive && ((valid >> pi) & 1u)) {
            const uint64_t h = bloom_hash(later[j]);
            const uint32_t* blk = s_blocks[pi] + static_cast<uint64_t>(bloom_block_of(h, s_nblocks[pi])) * 8;
            alive = bloom_test(blk, h, p.probes[pi].num_hashes);
          }
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, alive);
        __syncwarp();  // every lane has read its entry before any is overwritten
        if (alive) list[m + __popc(bal & lane_lt)] = static_cast<uint16_t>(r);
        m += __popc(bal);
        __syncwarp();
      }
      n_alive = m;
    }
    // (4) the slice's row ids, in order, into its part of the row list
    int32_t* dst = rowlist + start;
    for (int i = lane; i < n_alive; i += 32) dst[i] = static_cast<int32_t>(start + list[i]);
    if (lane == 0) {
      reinterpret_cast<uint32_t*>(p.tile_status)[sl] = static_cast<uint32_t>(n_alive);
      if (n_alive > 0) atomicAdd(range_totals + sl / kGatherSlices, static_cast<unsigned int>(n_alive));
    }
    __syncwarp();  // the list is rewritten by the warp's next slice
  }
}

// Pass 2: ranges of kGatherSlices consecutive slices. Pass 1 also added
// each slice's count into its range's total, so a CTA learns the rows of all
// earlier ranges by summing their totals (no ordering between CTAs), scans
// its own slices' counts, then moves every selected row of its range in one
// parallel pass (row ids in order in each slice's part of the row-id buffer)
// to the output. The CTA holding the last range records the total.
__global__ void __launch_bounds__(kSelThreads) select_gather_kernel(const __grid_constant__ SelectParams p,
                                                                   const int32_t* rowlist, int32_t* out_rowids,
                                                                   const unsigned int* __restrict__ range_totals) {
  __shared__ int s_w[kSelThreads / 32 + 1];
  __shared__ int s_pref[kSelThreads + 1];
  const int64_t n_rows = clamp_rows(p.n_dev, p.n_rows);
  const int64_t n_tiles = (n_rows + kPwRows - 1) / kPwRows;
  const int64_t n_ranges = (n_tiles + kGatherSlices - 1) / kGatherSlices;
  const uint32_t* counts = reinterpret_cast<const uint32_t*>(p.tile_status);  // uint32, from select_probe_kernel
  for (int64_t r = blockIdx.x; r < n_ranges; r += gridDim.x) {
    int64_t part = 0;
    for (int64_t q = threadIdx.x; q < r; q += kSelThreads) part += range_totals[q];
    int before;
    (void)block_exclusive_sum<kSelThreads>(static_cast<int>(part), &before, s_w);
    __syncthreads();  // s_w is reused
    const int64_t t0 = r * kGatherSlices;
    const int64_t t1 = t0 + kGatherSlices < n_tiles ? t0 + kGatherSlices : n_tiles;
    const int nt = static_cast<int>(t1 - t0);
    const int c = threadIdx.x < nt ? static_cast<int>(counts[t0 + threadIdx.x]) : 0;
    int range_total;
    const int excl = block_exclusive_sum<kSelThreads>(c, &range_total, s_w);
    if (threadIdx.x < nt) s_pref[threadIdx.x] = excl;
    if (threadIdx.x == 0) s_pref[nt] = range_total;
    __syncthreads();
    const int64_t base = before;
    for (int i = threadIdx.x; i < range_total; i += kSelThreads) {
      int lo = 0, hi = nt - 1;  // last slice of the range whose first output is <= i
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_pref[mid] <= i) lo = mid;
        else hi = mid - 1;
      }
      const int32_t row = rowlist[(t0 + lo) * kPwRows + (i - s_pref[lo])];
      const int64_t o = base + i;
      for (int j = 0; j < p.n_out; ++j) {
        const OutCol& oc = p.outs[j];
        if (oc.width == 8)
          static_cast<long long*>(oc.dst)[o] = __ldg(static_cast<const long long*>(oc.src) + row);
        else
          static_cast<int*>(oc.dst)[o] = __ldg(static_cast<const int*>(oc.src) + row);
      }
      if (out_rowids != nullptr) out_rowids[o] = row;
    }
    if (r == n_ranges - 1 && threadIdx.x == 0) p.status->value = base + range_total;
    __syncthreads();  // s_pref and s_w are rewritten for the next range
  }
}

using ProbeKernel = void (*)(SelectParams, StreamPred, int32_t*, unsigned int*);

// The instantiation for a predicate (or none) and a number of later probes.
ProbeKernel select_probe_fn(bool with_pred, int n_later) {
  const int k = n_later <= 3 ? n_later : 4;
  static const ProbeKernel table[2][5] = {
      {select_probe_kernel<false, 0>, select_probe_kernel<false, 1>, select_probe_kernel<false, 2>,
       select_probe_kernel<false, 3>, select_probe_kernel<false, -1>},
      {select_probe_kernel<true, 0>, select_probe_kernel<true, 1>, select_probe_kernel<true, 2>,
       select_probe_kernel<true, 3>, select_probe_kernel<true, -1>}};
  return table[with_pred ? 1 : 0][k];
}

int select_probe_blocks_per_sm(ProbeKernel fn, size_t dyn) {
  static std::mutex mu;
  static std::map<std::pair<const void*, size_t>, int> cache;
  static std::set<const void*> attr_set;
  std::lock_guard<std::mutex> lk(mu);
  const void* f = reinterpret_cast<const void*>(fn);
  const auto key = std::make_pair(f, dyn);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  if (!attr_set.count(f)) {
    GF_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSpMaxDynamic)));
    attr_set.insert(f);
  }
  int per_sm = 0;
  GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kPwThreads, dyn));
  cache[key] = per_sm;
  return per_sm;
}

// ---------------------------------------------------------------------------
// Compact selection for small inputs (dimension tables, small partitions).
// A launch over a few thousand rows is bound by instruction fetch and by the
// chain of dependent global accesses, not by bytes, so this kernel keeps its
// code and its parameter block small: leaves are (integer column op integer
// literal) with the comparison reduced to a 4-bit truth table over
// (value < literal, value == literal), filters are probed in global memory
// (they sit in L2) and a CTA whose grid covers every tile takes one ticket.
constexpr int kLiteThreads = 256;
constexpr int kLiteItems = 4;
constexpr int kLiteTile = kLiteThreads * kLiteItems;
constexpr int kLiteMaxLeaves = 8;
constexpr int kLiteMaxOut = 12;
constexpr int64_t kLiteMaxRows = int64_t{1} << 18;

struct LiteProbe {
  const uint32_t* blocks;
  const uint64_t* nblocks_dev;
  const int32_t* valid_dev;
  const void* key;
  uint32_t num_blocks;
  int8_t wide;
  int8_t num_hashes;
  int8_t valid;
  int8_t pad;
};

struct LiteOut {
  const void* src;
  void* dst;
  int32_t width;
  int32_t pad;
};

struct LiteParams {
  int64_t n_rows;
  const int64_t* n_dev;
  int32_t n_leaves;
  int32_t n_probes;
  int32_t n_out;
  int32_t pad;
  SimpleLeaf leaves[kLiteMaxLeaves];
  LiteProbe probes[kMaxBlooms];
  LiteOut outs[kLiteMaxOut];
  int32_t* out_rowids;
  uint64_t* tile_status;
  uint32_t* ticket;
  DevStatus* status;
};

// Rows [row0, row0 + 4) of an integer column; full: all four exist (and the
// column is 16-byte aligned), else only the rows in `mask` are read.
__device__ __forceinline__ void lite_load4(const void* col, bool wide, int64_t row0, uint32_t mask, bool full,
                                           int64_t v[kLiteItems]) {
  if (wide) {
    const long long* q = static_cast<const long long*>(col) + row0;
    if (full) {
      const longlong2 a = __ldg(reinterpret_cast<const longlong2*>(q));
      const longlong2 b = __ldg(reinterpret_cast<const longlong2*>(q) + 1);
      v[0] = a.x;
      v[1] = a.y;
      v[2] = b.x;
      v[3] = b.y;
    } else {
#pragma unroll
      for (int k = 0; k < kLiteItems; ++k) v[k] = ((mask >> k) & 1u) ? __ldg(q + k) : 0;
    }
  } else {
    const int* q = static_cast<const int*>(col) + row0;
    if (full) {
      const int4 a = __ldg(reinterpret_cast<const int4*>(q));
      v[0] = a.x;
      v[1] = a.y;
      v[2] = a.z;
      v[3] = a.w;
    } else {
#pragma unroll
      for (int k = 0; k < kLiteItems; ++k) v[k] = ((mask >> k) & 1u) ? __ldg(q + k) : 0;
    }
  }
}

__global__ void __launch_bounds__(kLiteThreads) select_lite_kernel(const __grid_constant__ LiteParams p) {
  __shared__ int s_warp[kLiteThreads / 32 + 1];
  __shared__ uint32_t s_tile;
  __shared__ uint64_t s_base;
  const int64_t n_rows = clamp_rows(p.n_dev, p.n_rows);
  const int64_t n_tiles = (n_rows + kLiteTile - 1) / kLiteTile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(p.ticket, 1u);
    __syncthreads();
    const int64_t tile = s_tile;
    if (tile >= n_tiles) break;
    const int64_t row0 = tile * kLiteTile + static_cast<int64_t>(threadIdx.x) * kLiteItems;
    const int64_t rem = n_rows - row0;
    const bool full = rem >= kLiteItems;
    uint32_t mask = full ? 0xFu : (rem <= 0 ? 0u : (1u << rem) - 1u);

    // predicate: AND over clauses of OR over their leaves
    if (p.n_leaves > 0 && mask != 0) {
      uint32_t all = mask, any = 0;
#pragma unroll 1
      for (int l = 0; l < p.n_leaves; ++l) {
        const SimpleLeaf& L = p.leaves[l];
        if (L.clause_start && l > 0) {
          all &= any;
          any = 0;
        }
        int64_t v[kLiteItems];
        lite_load4(L.col, L.wide, row0, mask, full, v);
#pragma unroll
        for (int k = 0; k < kLiteItems; ++k) {
          const uint32_t idx = (static_cast<uint32_t>(v[k] < L.lit) << 1) | static_cast<uint32_t>(v[k] == L.lit);
          any |= ((static_cast<uint32_t>(L.truth) >> idx) & 1u) << k;
        }
      }
      mask = all & any;
    }

    // bloom probes
#pragma unroll 1
    for (int pi = 0; pi < p.n_probes; ++pi) {
      const LiteProbe& pr = p.probes[pi];
      const bool valid = pr.valid_dev ? (*pr.valid_dev != 0) : (pr.valid != 0);
      if (!valid || mask == 0) continue;
      const uint32_t nb = pr.nblocks_dev ? static_cast<uint32_t>(*pr.nblocks_dev) : pr.num_blocks;
      int64_t keys[kLiteItems];
      lite_load4(pr.key, pr.wide, row0, mask, full, keys);
      uint32_t keep = 0;
#pragma unroll
      for (int k = 0; k < kLiteItems; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const uint64_t h = bloom_hash(keys[k]);
        const uint4* words = reinterpret_cast<const uint4*>(pr.blocks + static_cast<uint64_t>(bloom_block_of(h, nb)) * 8);
        const uint4 lo = __ldg(words);
        const uint4 hi = __ldg(words + 1);
        const uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        keep |= static_cast<uint32_t>(bloom_test(w, h, pr.num_hashes)) << k;
      }
      mask &= keep;
    }

    // rank (block scan + decoupled look-back), then move the selected rows
    const int cnt = __popc(mask);
    int tile_total;
    const int excl = block_exclusive_sum<kLiteThreads>(cnt, &tile_total, s_warp);
    if (threadIdx.x < 32) {
      const uint64_t b = lookback_exclusive(p.tile_status, tile, static_cast<uint64_t>(tile_total), p.status);
      if (threadIdx.x == 0) s_base = b;
    }
    __syncthreads();
    const int64_t base = static_cast<int64_t>(s_base);
    if (mask != 0) {
      const int64_t out0 = base + excl;
      // four output columns at a time: their loads (16-byte vectors on full
      // groups) in flight together, then the compacted stores
#pragma unroll 1
      for (int j0 = 0; j0 < p.n_out; j0 += 4) {
        int64_t v[4][kLiteItems];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj)
          if (j0 + jj < p.n_out) lite_load4(p.outs[j0 + jj].src, p.outs[j0 + jj].width == 8, row0, mask, full, v[jj]);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          if (j0 + jj >= p.n_out) break;
          const LiteOut& oc = p.outs[j0 + jj];
          int o = 0;
          if (oc.width == 8) {
#pragma unroll
            for (int k = 0; k < kLiteItems; ++k)
              if ((mask >> k) & 1u) static_cast<long long*>(oc.dst)[out0 + o++] = v[jj][k];
          } else {
#pragma unroll
            for (int k = 0; k < kLiteItems; ++k)
              if ((mask >> k) & 1u) static_cast<int*>(oc.dst)[out0 + o++] = static_cast<int>(v[jj][k]);
          }
        }
      }
      if (p.out_rowids != nullptr) {
        int o = 0;
#pragma unroll
        for (int k = 0; k < kLiteItems; ++k)
          if ((mask >> k) & 1u) p.out_rowids[out0 + o++] = static_cast<int32_t>(row0 + k);
      }
    }
    if (tile == n_tiles - 1 && threadIdx.x == 0) p.status->value = base + tile_total;
    if (static_cast<int64_t>(gridDim.x) >= n_tiles) break;  // every tile was claimed by the first tickets
    __syncthreads();
  }
}

// The compact kernel's parameters for a select, or false when the select
// needs the general kernel (a leaf that is not integer column vs integer
// literal, an empty clause, too many leaves or outputs, or a column that is
// not 16-byte aligned).
bool lite_params(const SelectParams& p, LiteParams& lp) {
  std::memset(&lp, 0, sizeof(lp));
  auto aligned = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  if (!simple_leaves(p, lp.leaves, kLiteMaxLeaves, &lp.n_leaves)) return false;
  lp.n_probes = p.n_probes;
  for (int pi = 0; pi < p.n_probes; ++pi) {
    const BloomDev& b = p.probes[pi];
    const DevCol& dc = p.cols[b.col];
    if (!aligned(dc.data)) return false;
    LiteProbe& o = lp.probes[pi];
    o.blocks = b.blocks;
    o.nblocks_dev = b.nblocks_dev;
    o.valid_dev = b.valid_dev;
    o.key = dc.data;
    o.num_blocks = b.num_blocks;
    o.wide = dc.type == CT_I64 ? 1 : 0;
    o.num_hashes = b.num_hashes;
    o.valid = b.valid;
  }
  if (p.n_out > kLiteMaxOut) return false;
  lp.n_out = p.n_out;
  for (int j = 0; j < p.n_out; ++j) {
    if (!aligned(p.outs[j].src)) return false;  // read with 16-byte vectors
    lp.outs[j].src = p.outs[j].src;
    lp.outs[j].dst = p.outs[j].dst;
    lp.outs[j].width = p.outs[j].width;
  }
  lp.n_rows = p.n_rows;
  lp.n_dev = p.n_dev;
  lp.out_rowids = p.out_rowids;
  return true;
}

int select_lite_blocks_per_sm() {
  static const int per_sm = [] {
    int v = 0;
    GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, select_lite_kernel, kLiteThreads, 0));
    return v < 1 ? 1 : v;
  }();
  return per_sm;
}

}  // namespace

TupleSetPtr select_rows(const TupleSet& in, const CompiledPredicate* pred, const std::vector<BloomProbe>& probes,
                        const std::vector<std::string>& project, bool all_columns, cudaStream_t s,
                        SelectStats* stats) {
  const int64_t n = in.num_rows();  // exact, or the capacity of a deferred input
  if (n >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "a TupleSet passed to select must have fewer than 2^31 rows");
  if (static_cast<int>(probes.size()) > kMaxBlooms) fail(GFPDB_EUNSUPPORTED, "too many bloom probes in one select");

  auto* pp = new SelectParams;  // large; keep off the stack
  std::unique_ptr<SelectParams> holder(pp);
  SelectParams& p = *pp;
  std::memset(&p, 0, sizeof(p));
  p.n_rows = n;
  p.n_dev = in.rows_dev();

  ColumnSlots slots;
  if (pred != nullptr) {
    p.prog = pred->prog;
    slots = pred->slots;
  }
  // bloom key columns take slots after the predicate's
  std::vector<int> probe_slot;
  for (auto& pr : probes) {
    int ci = in.require_column(pr.column);
    DType t = in.field(ci).type;
    if (t != DType::Int32 && t != DType::Int64 && t != DType::Date32)
      fail(GFPDB_EUNSUPPORTED, "bloom key column '" + pr.column + "' must be an integer column");
    probe_slot.push_back(slots.slot_for(pr.column, t));
  }
  bind_columns(slots, in, p.cols, kMaxCols);
  p.n_cols = static_cast<int32_t>(slots.names.size());
  bool aligned = true;
  for (int i = 0; i < p.n_cols; ++i)
    if ((reinterpret_cast<uintptr_t>(p.cols[i].data) & 15u) != 0) aligned = false;
  p.aligned = aligned ? 1 : 0;

  // Shared-memory slots for the filters: an exact filter gets its whole size
  // while the budget lasts; a filter whose size is only known on the device
  // gets up to kDeferredBloomSlot bytes and is staged if it turns out to fit.
  constexpr int kDeferredBloomSlot = 16 * 1024;
  int smem_words = 0;
  p.n_probes = static_cast<int32_t>(probes.size());
  for (size_t i = 0; i < probes.size(); ++i) {
    const auto& bf = *probes[i].bloom;
    BloomDev& b = p.probes[i];
    b.blocks = bf.blocks->as<uint32_t>();
    if (bf.num_blocks >= (int64_t{1} << 32)) fail(GFPDB_EUNSUPPORTED, "bloom filter too large");
    b.num_blocks = static_cast<uint32_t>(bf.num_blocks);
    b.nblocks_dev = bf.nblocks_dev;
    b.valid_dev = bf.valid_dev;
    b.col = static_cast<int16_t>(probe_slot[i]);
    b.num_hashes = static_cast<int8_t>(bf.num_hashes);
    b.valid = bf.valid ? 1 : 0;
    int64_t words = bf.num_blocks * 8;
    if (bf.nblocks_dev != nullptr && words * 4 > kDeferredBloomSlot) words = kDeferredBloomSlot / 4;
    if ((bf.valid || bf.valid_dev) && (smem_words + words) * 4 <= kBloomSmemBudget) {
      b.smem_word = smem_words;
      b.smem_cap_words = static_cast<int32_t>(words);
      smem_words += static_cast<int>(words);
    } else {
      b.smem_word = -1;
    }
  }
  p.smem_words = smem_words;

  // outputs
  std::vector<std::string> out_names = project;
  if (all_columns) {
    out_names.clear();
    for (auto& f : in.fields()) out_names.push_back(f.name);
  }
  std::vector<Field> out_fields;
  std::vector<ColumnPtr> out_cols(out_names.size());
  std::vector<BufferPtr> out_bufs(out_names.size());
  bool need_rowids = false;
  for (size_t j = 0; j < out_names.size(); ++j) {
    int ci = in.require_column(out_names[j]);
    out_fields.push_back(in.field(ci));
    const auto& c = in.column(ci);
    if (c->type == DType::Utf8) {
      need_rowids = true;
      continue;
    }
    const int w = dtype_width(c->type);
    out_bufs[j] = make_buffer(n * w, s);
    OutCol& oc = p.outs[p.n_out++];
    oc.src = c->data;
    oc.dst = out_bufs[j]->data();
    oc.width = w;
    oc.aligned = (reinterpret_cast<uintptr_t>(c->data) & 15u) == 0 ? 1 : 0;
  }
  BufferPtr rowids;
  if (need_rowids) {
    rowids = make_buffer(n * 4, s);
    p.out_rowids = rowids->as<int32_t>();
  }

  // small inputs of the simple shapes take the compact kernel (its tiles are
  // smaller, so the tile-status array is sized for them)
  LiteParams lp;
  const bool lite = n <= kLiteMaxRows && lite_params(p, lp);
  // probe-only selections over large inputs take the two-pass kernels (their
  // unit is a warp's 256-row slice)
  // (probe chains, and predicates of simple leaves, with or without probes)
  StreamPred spred{};
  const bool two_pass = !lite && n >= kSpMinRows && simple_leaves(p, spred.leaves, kSimpleMaxLeaves, &spred.n_leaves) &&
                        (p.n_probes > 0 || spred.n_leaves > 0);
  const int64_t unit = lite ? kLiteTile : two_pass ? kPwRows : kSelTile;
  const int64_t n_tiles = (n + unit - 1) / unit;  // upper bound
  p.n_tiles = n_tiles;
  auto scratch = make_filled(sizeof(DevStatus) + 64 + n_tiles * 8, 0, s);
  char* sb = scratch->as<char>();
  p.status = reinterpret_cast<DevStatus*>(sb);
  p.ticket = reinterpret_cast<uint32_t*>(sb + sizeof(DevStatus));
  p.tile_status = reinterpret_cast<uint64_t*>(sb + sizeof(DevStatus) + 64);

  // Algorithmic bytes: every evaluated column read once over all rows, the
  // selected rows of the other projected columns read once, every projected
  // value written once.
  double read_all = 0, proj_read = 0, proj_write = 0;
  for (int i = 0; i < p.n_cols; ++i) read_all += dtype_width(static_cast<DType>(p.cols[i].type));
  for (int j = 0; j < p.n_out; ++j) {
    proj_write += p.outs[j].width;
    bool evaluated = false;
    for (int i = 0; i < p.n_cols; ++i) evaluated |= p.cols[i].data == p.outs[j].src;
    if (!evaluated) proj_read += p.outs[j].width;
  }
  if (n_tiles > 0 && lite) {
    lp.tile_status = p.tile_status;
    lp.ticket = p.ticket;
    lp.status = p.status;
    const int64_t cap = static_cast<int64_t>(num_sms()) * select_lite_blocks_per_sm();
    ProfScope prof("select_lite_kernel", s);
    select_lite_kernel<<<static_cast<int>(n_tiles < cap ? n_tiles : cap), kLiteThreads, 0, s>>>(lp);
    after_launch("select_lite_kernel");
    prof.stop(0);
    prof.set_bytes_model(p.n_dev, n, read_all, &p.status->value, proj_read + proj_write, scratch, in.rows_owner());
  } else if (n_tiles > 0 && two_pass) {
    // pass 1: probes; each slice's selected row ids into its part of rowlist
    // every filter that fits is staged (the layout stays within
    // kBloomSmemBudget, which is kSpMaxDynamic)
    const size_t dyn = static_cast<size_t>(p.smem_words) * 4;
    const bool with_pred = spred.n_leaves > 0;
    const ProbeKernel fn = select_probe_fn(with_pred, p.n_probes > 0 ? p.n_probes - 1 : 0);
    const int per_sm = select_probe_blocks_per_sm(fn, dyn);
    auto rowlist = make_buffer(n * 4, s);
    const int64_t n_ranges = (n_tiles + kGatherSlices - 1) / kGatherSlices;
    auto range_totals = make_filled(n_ranges * 4, 0, s);
    {
      const int64_t want = (n_tiles + kPwThreads / 32 - 1) / (kPwThreads / 32);
      const int64_t cap = static_cast<int64_t>(num_sms()) * (per_sm > 0 ? per_sm : 1);
      ProfScope prof("select_probe_kernel", s);
      const int grid = static_cast<int>(want < cap ? want : cap);
      fn<<<grid, kPwThreads, dyn, s>>>(p, spred, rowlist->as<int32_t>(), range_totals->as<unsigned int>());
      after_launch("select_probe_kernel");
      prof.stop(0);
      // the predicate's columns and the first probe's keys over all rows
      // (later probes' keys are read for survivors only and not counted)
      double per_row = 0;
      for (int l = 0; l < spred.n_leaves; ++l) {
        bool seen = false;
        for (int m = 0; m < l; ++m) seen |= spred.leaves[m].col == spred.leaves[l].col;
        if (!seen) per_row += spred.leaves[l].wide ? 8 : 4;
      }
      if (p.n_probes > 0) per_row += p.cols[p.probes[0].col].type == CT_I64 ? 8 : 4;
      prof.set_bytes_model(p.n_dev, n, per_row, &p.status->value, 4.0, scratch, in.rows_owner());
    }
    {
      // one CTA per range of kGatherSlices slices (grid-stride beyond four per SM)
      const int64_t cap = static_cast<int64_t>(num_sms()) * 4;
      ProfScope prof("select_gather_kernel", s);
      select_gather_kernel<<<static_cast<int>(n_ranges < 1 ? 1 : (n_ranges < cap ? n_ranges : cap)), kSelThreads, 0, s>>>(
          p, rowlist->as<int32_t>(), p.out_rowids, range_totals->as<unsigned int>());
      after_launch("select_gather_kernel");
      prof.stop(0);
      prof.set_bytes_model(nullptr, 0, 0, &p.status->value, 4.0 + proj_read + proj_write, scratch, in.rows_owner());
    }  // rowlist is freed stream-ordered, after the gather
  } else if (n_tiles > 0) {
    const size_t dyn = static_cast<size_t>(smem_words) * 4;
    const bool with_pred = p.prog.n_clauses > 0;
    {
      int per_sm = 0;
      ProfScope prof("select_kernel", s);
      per_sm = select_blocks_per_sm(with_pred, dyn);
      int64_t grid = static_cast<int64_t>(num_sms()) * per_sm;
      if (grid > n_tiles) grid = n_tiles;
      if (with_pred)
        select_kernel<true><<<static_cast<int>(grid), kSelThreads, dyn, s>>>(p);
      else
        select_kernel<false><<<static_cast<int>(grid), kSelThreads, dyn, s>>>(p);
      after_launch("select_kernel");
      prof.stop(0);
      prof.set_bytes_model(p.n_dev, n, read_all, &p.status->value, proj_read + proj_write, scratch,
                           in.rows_owner());
    }
  }

  const bool defer = deferred_mode() && !need_rowids && stats == nullptr;
  if (defer) {
    defer_check(scratch, p.status, "select");
    for (size_t j = 0; j < out_names.size(); ++j)
      out_cols[j] = make_fixed_column(out_fields[j].type, n, out_bufs[j]);
    return TupleSet::make_deferred(std::move(out_fields), std::move(out_cols), n, scratch, &p.status->value);
  }
  int64_t count = 0;
  if (n_tiles > 0) {
    DevStatus hs;
    GF_CUDA(cudaMemcpyAsync(&hs, p.status, sizeof(hs), cudaMemcpyDeviceToHost, s));
    sync(s);
    raise_device_status(hs, "select");
    count = hs.value;
  }
  for (size_t j = 0; j < out_names.size(); ++j) {
    if (out_fields[j].type == DType::Utf8) continue;
    out_cols[j] = make_fixed_column(out_fields[j].type, count, out_bufs[j]);
  }
  if (need_rowids) {
    std::vector<GatherSpec> specs;
    std::vector<size_t> which;
    for (size_t j = 0; j < out_names.size(); ++j) {
      if (out_fields[j].type != DType::Utf8) continue;
      specs.push_back(GatherSpec{in.column(in.require_column(out_names[j])).get(), rowids->as<int32_t>()});
      which.push_back(j);
    }
    auto g = gather_columns(specs, count, s);
    for (size_t k = 0; k < which.size(); ++k) out_cols[which[k]] = g[k];
  }
  if (stats) {
    stats->rows_in = n;
    stats->rows_out = count;
  }
  return TupleSet::make(std::move(out_fields), std::move(out_cols), count);
}

}  // namespace gfpdb

// ---------------------------------------------------------------------------
// Filter evaluation that allocates no device memory.
//
// Some callers cannot call cudaMalloc at all: engines that hand the library
// a fixed device arena and account for every byte of HBM themselves (a
// cudaMalloc would grow the device heap behind their back and can fail or
// stall while they hold the rest of the memory), and embedders whose device
// memory belongs to another runtime's allocator (a second allocator in the
// same process fragments and double-counts the pool). For them
// gfpdb_filter_evaluate_noalloc runs the same
// select_kernel with its scratch (the call's status block, the tile ticket
// and one look-back word per 2048-row tile) in the file-scope array below
// instead of a per-call allocation. The array is sized for
// kNoAllocMaxRows input rows (about 1 MiB) and, being a __device__ variable,
// lives on every GPU that loads this library until the process exits.
namespace gfpdb {
namespace {

constexpr int64_t kNoAllocMaxRows = int64_t{1} << 28;  // 268,435,456 rows
constexpr int64_t kNoAllocMaxTiles = kNoAllocMaxRows / kSelTile;
constexpr size_t kNoAllocHeader = 128;  // DevStatus (64 B) + ticket line (64 B)
constexpr size_t kNoAllocScratchBytes = kNoAllocHeader + static_cast<size_t>(kNoAllocMaxTiles) * 8;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch for each device, looked up once per
// device with that device current (host code only has a host-side stand-in
// for the symbol, which must never be passed to a kernel).
std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {};

void* noalloc_scratch_address(int device) {
  if (device < 0 || device >= 64) fail(GFPDB_EUNSUPPORTED, "device index above 63");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_addr[device] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) check_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_addr[device] = p;
  }
  return g_noalloc_addr[device];
}

int find_child(const ArrowSchema* schema, const char* name) {
  for (int64_t i = 0; i < schema->n_children; ++i) {
    const char* cn = schema->children[i]->name;
    if (cn != nullptr && std::strcmp(cn, name) == 0) return static_cast<int>(i);
  }
  return -1;
}

}  // namespace
}  // namespace gfpdb

extern "C" int32_t gfpdb_filter_evaluate_noalloc(const gfpdb_filter* filter, const ArrowSchema* in_schema,
                                                 const ArrowDeviceArray* in, const char* const* project_columns,
                                                 int32_t n_project, void* const* out_columns, int64_t* out_num_rows,
                                                 void* stream) {
  using namespace gfpdb;
  return guarded([&] {
    if (filter == nullptr || in_schema == nullptr || in == nullptr || out_num_rows == nullptr)
      fail(GFPDB_EINVAL, "null argument");
    if (n_project < 0 || (n_project > 0 && (project_columns == nullptr || out_columns == nullptr)))
      fail(GFPDB_EINVAL, "project_columns and out_columns must list the output columns");
    if (n_project > kMaxCols) fail(GFPDB_EUNSUPPORTED, "too many output columns");
    if (in_schema->format == nullptr || std::strcmp(in_schema->format, "+s") != 0)
      fail(GFPDB_EINVAL, "a TupleSet schema must be a struct (format \"+s\")");
    if (in->device_type != ARROW_DEVICE_CUDA)
      fail(GFPDB_EINVAL, "gfpdb_filter_evaluate_noalloc needs device-resident input (ARROW_DEVICE_CUDA)");
    const ArrowArray& arr = in->array;
    if (arr.release == nullptr) fail(GFPDB_EINVAL, "released ArrowArray");
    if (arr.n_children != in_schema->n_children) fail(GFPDB_EINVAL, "ArrowArray child count does not match the schema");
    const int64_t n = arr.length;
    if (n < 0 || arr.offset < 0) fail(GFPDB_EINVAL, "negative row count or offset");
    if (n > kNoAllocMaxRows)
      fail(GFPDB_EINVAL, "gfpdb_filter_evaluate_noalloc: " + std::to_string(n) + " rows exceed its maximum of " +
                             std::to_string(kNoAllocMaxRows) + " rows");
    if (arr.null_count > 0) fail(GFPDB_EUNSUPPORTED, "struct-level nulls are not supported");
    // The checks import_tupleset makes for gfpdb_filter_evaluate, on every
    // column the call reads: long enough for the struct's offset + length,
    // the buffer count of its type, no nulls.
    auto bound_child = [&](int ci, DType t, const std::string& name) -> const ArrowArray* {
      const ArrowArray* c = arr.children[ci];
      if (c == nullptr || c->release == nullptr) fail(GFPDB_EINVAL, "column '" + name + "' is missing or released");
      if (c->offset < 0 || c->length < arr.offset + n)
        fail(GFPDB_EINVAL, "column '" + name + "' is shorter than the struct");
      if (c->n_buffers != (t == DType::Utf8 ? 3 : 2))
        fail(GFPDB_EINVAL, "column '" + name + "' has the wrong number of buffers for its type");
      if (c->null_count != 0 && c->buffers[0] != nullptr)
        fail(GFPDB_EUNSUPPORTED, "column '" + name + "' has nulls; nullable inputs are not supported");
      return c;
    };
    int device = 0;
    GF_CUDA(cudaGetDevice(&device));
    // First call on this device: look up the scratch address (no allocation).
    void* scratch = noalloc_scratch_address(device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    SelectParams p;
    std::memset(&p, 0, sizeof(p));
    p.n_rows = n;
    const CompiledPredicate& pred = filter->pred;
    p.prog = pred.prog;
    // Bind the predicate's columns straight from the Arrow structures.
    bool aligned = true;
    for (size_t i = 0; i < pred.slots.names.size(); ++i) {
      const int ci = find_child(in_schema, pred.slots.names[i].c_str());
      if (ci < 0) fail(GFPDB_EINVAL, "column '" + pred.slots.names[i] + "' not found in TupleSet");
      const DType t = dtype_from_format(in_schema->children[ci]->format);
      if (t != pred.slots.types[i]) fail(GFPDB_EINVAL, "column '" + pred.slots.names[i] + "' changed type");
      const ArrowArray* c = bound_child(ci, t, pred.slots.names[i]);
      const int64_t off = c->offset + arr.offset;
      if (t == DType::Utf8) {
        p.cols[i].offsets = static_cast<const int32_t*>(c->buffers[1]) + off;
        p.cols[i].data = c->buffers[2];
      } else {
        p.cols[i].data = static_cast<const char*>(c->buffers[1]) + off * dtype_width(t);
        if ((reinterpret_cast<uintptr_t>(p.cols[i].data) & 15u) != 0) aligned = false;
      }
      p.cols[i].type = static_cast<int32_t>(t);
    }
    p.n_cols = static_cast<int32_t>(pred.slots.names.size());
    p.aligned = aligned ? 1 : 0;
    // Outputs: fixed-width columns written straight into the caller's buffers.
    for (int32_t j = 0; j < n_project; ++j) {
      if (project_columns[j] == nullptr || out_columns[j] == nullptr) fail(GFPDB_EINVAL, "null output column");
      const int ci = find_child(in_schema, project_columns[j]);
      if (ci < 0) fail(GFPDB_EINVAL, std::string("column '") + project_columns[j] + "' not found in TupleSet");
      const DType t = dtype_from_format(in_schema->children[ci]->format);
      if (t == DType::Utf8) fail(GFPDB_EUNSUPPORTED, "utf8 outputs need allocation; use gfpdb_filter_evaluate");
      const ArrowArray* c = bound_child(ci, t, project_columns[j]);
      OutCol& oc = p.outs[p.n_out++];
      oc.src = static_cast<const char*>(c->buffers[1]) + (c->offset + arr.offset) * dtype_width(t);
      oc.dst = out_columns[j];
      oc.width = dtype_width(t);
      oc.aligned = (reinterpret_cast<uintptr_t>(oc.src) & 15u) == 0 ? 1 : 0;
    }
    const int64_t n_tiles = (n + kSelTile - 1) / kSelTile;
    p.n_tiles = n_tiles;
    char* sb = static_cast<char*>(scratch);
    p.status = reinterpret_cast<DevStatus*>(sb);
    p.ticket = reinterpret_cast<uint32_t*>(sb + sizeof(DevStatus));
    p.tile_status = reinterpret_cast<uint64_t*>(sb + kNoAllocHeader);
    // The array keeps the previous call's contents: clear the status block,
    // the ticket and this call's tile words.
    GF_CUDA(cudaMemsetAsync(sb, 0, kNoAllocHeader + static_cast<size_t>(n_tiles) * 8, s));
    int64_t count = 0;
    if (n_tiles > 0) {
      int64_t grid = static_cast<int64_t>(num_sms()) * select_blocks_per_sm(true, 0);
      if (grid > n_tiles) grid = n_tiles;
      select_kernel<true><<<static_cast<int>(grid), kSelThreads, 0, s>>>(p);
      after_launch("select_kernel");
      DevStatus hs;
      GF_CUDA(cudaMemcpyAsync(&hs, p.status, sizeof(hs), cudaMemcpyDeviceToHost, s));
      GF_CUDA(cudaStreamSynchronize(s));
      raise_device_status(hs, "select");
      count = hs.value;
    }
    *out_num_rows = count;
  });
}
