// Hash group-by with exact integer aggregates.
//
// Replaces the Arrow hash aggregate (hash_sum / hash_count / hash_min_max)
// that GroupArrowKernel drives (fpdb-executor/src/physical/group/GroupArrowKernel.cpp:127-154,
// fpdb-executor/src/physical/aggregate/function/Sum.cpp:63-74, Count.cpp:91-104)
// and the native GroupKernel (fpdb-executor/src/physical/group/GroupKernel.cpp:263-300).
//
// Keys: up to two key columns packed into one 64-bit word (32 bits per int32 /
// date32 column, 64 bits for one int64 column); a utf8 key column is first
// mapped to dense int32 codes by a device string dictionary that persists
// across batches. Wider keys (three to eight columns, or two whose widths add
// up to more than 64 bits) are written as fixed-width records of their
// values (utf8 columns by their codes) and mapped to dense int32 codes by the
// same dictionary over the records, and the table groups by that code; the
// key columns are recovered from the records at finalisation. The all-ones
// word marks an empty slot, so the one key that packs to all-ones gets a
// dedicated extra slot at index `capacity`.
//
// Aggregation: each CTA first folds its rows into a shared-memory table
// (64-bit atomicCAS on keys, 64-bit atomics on accumulators) and merges the
// table into the global open-addressing table once at the end, so
// low-cardinality group-bys (a handful to a few thousand groups) cost one
// global atomic per group per CTA rather than per row. Rows whose key does
// not fit the shared table go straight to the global table. New groups are
// counted per CTA in shared memory and added to the table's count once per
// CTA. Integer sums are 64-bit two's-complement additions, which are
// associative and commutative, so results are bit-exact whatever order the
// atomics land in.
//
// Table size: at most half full for an upper bound on the groups (groups so
// far plus the batch's rows). A large batch whose rows are known on the host
// is first counted with a HyperLogLog sketch of its keys, and the table is
// sized for that estimate instead: a batch of 20M rows over 1.8M distinct
// keys gets 4M slots (96 MB with two accumulators) rather than 64M (1.5 GB)
// to fill and to scan at finalisation.
#include <cmath>
#include <cstring>
#include <vector>

#include "eval.cuh"
#include "launch.h"

namespace gfpdb {

namespace {

constexpr int kGroupThreads = 256;
constexpr int kGroupSmemSlotsMax = 1024;  // slots of a CTA's shared-memory table
constexpr int kGroupSmemProbes = 4;       // shared-memory slots a row tries before the global table
constexpr uint32_t kDictSpinLimit = 1u << 20;

struct AccDev {
  int8_t fn;  // AGG_SUM / AGG_COUNT / AGG_MIN / AGG_MAX / AGG_COUNT_STAR
  int8_t vt;
  int16_t pad;
  int32_t pad2;
  Operand in;
};

struct GroupParams {
  int64_t n_rows;          // exact, or the capacity when n_dev is set
  const int64_t* n_dev;    // device row count of a deferred batch
  int32_t n_keys;
  int32_t n_acc;
  int32_t key_bits[2];
  DevCol key_cols[2];
  AccDev acc[kMaxAggs];
  DevCol cols[kMaxCols];
  uint64_t* keys;
  unsigned long long* accs;
  uint64_t mask;
  int32_t use_smem;
  int32_t sm_slots;
  DevStatus* st;  // aux[0]: groups claimed, aux[1]: special slot used
  Program prog;
};

// A batch's columns are read once: streaming loads (evict-first) leave the
// L2 to the table, which every row revisits.
__device__ __forceinline__ int64_t load_int_stream(const DevCol& c, int64_t row) {
  if (c.type == CT_I64) return __ldcs(static_cast<const long long*>(c.data) + row);
  return __ldcs(static_cast<const int*>(c.data) + row);
}

__device__ __forceinline__ uint64_t pack_key(const GroupParams& p, int64_t row) {
  if (p.n_keys == 0) return 0;  // a non-grouped aggregate: one group
  if (p.n_keys == 1) {
    const int64_t v = load_int_stream(p.key_cols[0], row);
    return p.key_bits[0] == 64 ? static_cast<uint64_t>(v) : static_cast<uint64_t>(static_cast<uint32_t>(v));
  }
  const uint32_t a = static_cast<uint32_t>(load_int_stream(p.key_cols[0], row));
  const uint32_t b = static_cast<uint32_t>(load_int_stream(p.key_cols[1], row));
  return (static_cast<uint64_t>(a) << 32) | b;
}

// Identity of each accumulator: 0 for sums and counts, +inf / INT64_MAX for
// MIN, -inf / INT64_MIN for MAX (as bit patterns).
__device__ __forceinline__ unsigned long long acc_init(int fn, int vt) {
  if (fn == AGG_MIN) return vt == VT_F64 ? 0x7ff0000000000000ull : static_cast<unsigned long long>(INT64_MAX);
  if (fn == AGG_MAX) return vt == VT_F64 ? 0xfff0000000000000ull : static_cast<unsigned long long>(INT64_MIN);
  return 0ull;
}

__device__ __forceinline__ void acc_combine(unsigned long long* addr, int fn, int vt, unsigned long long v) {
  switch (fn) {
    case AGG_SUM:
      if (vt == VT_F64) atomicAdd(reinterpret_cast<double*>(addr), __longlong_as_double(static_cast<long long>(v)));
      else atomicAdd(addr, v);
      break;
    case AGG_COUNT:
    case AGG_COUNT_STAR: atomicAdd(addr, v); break;
    case AGG_MIN:
    case AGG_MAX: {
      if (vt == VT_F64) {
        const double x = __longlong_as_double(static_cast<long long>(v));
        unsigned long long old = *reinterpret_cast<volatile unsigned long long*>(addr);
        for (;;) {
          const double cur = __longlong_as_double(static_cast<long long>(old));
          const bool better = fn == AGG_MIN ? x < cur : x > cur;
          if (!better) break;
          const unsigned long long prev = atomicCAS(addr, old, v);
          if (prev == old) break;
          old = prev;
        }
      } else if (fn == AGG_MIN) {
        atomicMin(reinterpret_cast<long long*>(addr), static_cast<long long>(v));
      } else {
        atomicMax(reinterpret_cast<long long*>(addr), static_cast<long long>(v));
      }
      break;
    }
  }
}

// Global slot of a key that is not the all-ones word, continuing from its
// home slot `slot` whose content `s` the caller has already read; claims an
// empty slot for a new key. Returns UINT64_MAX (and raises GFPDB_ENOMEM) if
// the table is full.
__device__ __forceinline__ uint64_t global_slot_from(const GroupParams& p, uint64_t key, uint64_t slot, uint64_t s,
                                                     unsigned long long* claims) {
  for (uint64_t i = 0; i <= p.mask; ++i) {
    if (i > 0) s = *reinterpret_cast<volatile uint64_t*>(p.keys + slot);
    if (s == kEmptySlot) {
      s = atomicCAS(reinterpret_cast<unsigned long long*>(p.keys + slot), static_cast<unsigned long long>(kEmptySlot),
                    static_cast<unsigned long long>(key));
      if (s == kEmptySlot) {
        atomicAdd(claims, 1ull);
        return slot;
      }
    }
    if (s == key) return slot;
    slot = (slot + 1) & p.mask;
  }
  raise_status(p.st, GFPDB_ENOMEM, 20);
  return UINT64_MAX;
}

// The all-ones key has its own slot at index capacity.
__device__ __forceinline__ uint64_t special_slot(const GroupParams& p) {
  if (atomicExch(reinterpret_cast<unsigned long long*>(&p.st->aux[1]), 1ull) == 0ull)
    atomicAdd(reinterpret_cast<unsigned long long*>(&p.st->aux[0]), 1ull);
  return p.mask + 1;
}

// `claims` counts the groups this call creates: a CTA's shared-memory
// counter, added to the table's count once per CTA (one global address
// taking an atomic per new group would serialise the L2 on it).
__device__ __forceinline__ uint64_t global_slot(const GroupParams& p, uint64_t key, unsigned long long* claims) {
  if (key == kEmptySlot) return special_slot(p);
  const uint64_t slot = hash_key(static_cast<int64_t>(key)) & p.mask;
  return global_slot_from(p, key, slot, *reinterpret_cast<volatile uint64_t*>(p.keys + slot), claims);
}

__device__ __forceinline__ unsigned long long row_value(const GroupParams& p, const AccDev& a, int64_t row) {
  if (a.fn == AGG_COUNT || a.fn == AGG_COUNT_STAR) return 1ull;
  if (a.in.kind == OPND_COL) {  // a plain column (float64 as its bits), streamed
    const DevCol& c = p.cols[a.in.col];
    if (c.type == CT_I64 || c.type == CT_F64)
      return static_cast<unsigned long long>(__ldcs(static_cast<const long long*>(c.data) + row));
    return static_cast<unsigned long long>(static_cast<int64_t>(__ldcs(static_cast<const int*>(c.data) + row)));
  }
  return static_cast<unsigned long long>(operand_row(p.prog, p.cols, a.in, row, p.st));
}

__global__ void __launch_bounds__(kGroupThreads) group_update_kernel(const __grid_constant__ GroupParams p) {
  extern __shared__ unsigned long long s_mem[];
  __shared__ uint16_t s_occ[kGroupSmemSlotsMax];  // the occupied slots, listed for the merge
  __shared__ int s_scan[kGroupThreads / 32 + 1];
  uint64_t* s_keys = reinterpret_cast<uint64_t*>(s_mem);
  unsigned long long* s_acc = s_mem + p.sm_slots;
  const int sm_mask = p.sm_slots - 1;
  const int64_t n_rows = clamp_rows(p.n_dev, p.n_rows);
  // A grid sized for a capacity can be far larger than the rows that arrive:
  // CTAs without rows leave before touching shared memory (uniform per CTA).
  if (static_cast<int64_t>(blockIdx.x) * kGroupThreads >= n_rows) return;
  __shared__ unsigned long long s_claims;
  if (threadIdx.x == 0) s_claims = 0;
  if (p.use_smem) {
    for (int i = threadIdx.x; i < p.sm_slots; i += kGroupThreads) {
      s_keys[i] = kEmptySlot;
      for (int a = 0; a < p.n_acc; ++a) s_acc[i * p.n_acc + a] = acc_init(p.acc[a].fn, p.acc[a].vt);
    }
  }
  __syncthreads();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kGroupThreads;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * kGroupThreads + threadIdx.x; r < n_rows; r += stride) {
    const uint64_t key = pack_key(p, r);
    int found = -1;
    if (p.use_smem && key != kEmptySlot) {
      // A short probe run: with few groups the table is sparse and a key is
      // found or placed in a step or two; with many groups (high-cardinality
      // keys) the table is soon full and a longer run only delays the row's
      // trip to the global table.
      int slot = static_cast<int>(hash_key(static_cast<int64_t>(key)) & sm_mask);
      for (int i = 0; i < kGroupSmemProbes; ++i) {
        uint64_t s = *reinterpret_cast<volatile uint64_t*>(s_keys + slot);
        if (s == kEmptySlot) {
          s = atomicCAS(reinterpret_cast<unsigned long long*>(s_keys + slot),
                        static_cast<unsigned long long>(kEmptySlot), static_cast<unsigned long long>(key));
          if (s == kEmptySlot) s = key;
        }
        if (s == key) {
          found = slot;
          break;
        }
        slot = (slot + 1) & sm_mask;
      }
    }
    if (found >= 0) {
      for (int a = 0; a < p.n_acc; ++a)
        acc_combine(s_acc + found * p.n_acc + a, p.acc[a].fn, p.acc[a].vt, row_value(p, p.acc[a], r));
    } else {
      const uint64_t g = global_slot(p, key, &s_claims);
      if (g != UINT64_MAX)
        for (int a = 0; a < p.n_acc; ++a)
          acc_combine(p.accs + g * p.n_acc + a, p.acc[a].fn, p.acc[a].vt, row_value(p, p.acc[a], r));
    }
  }
  if (p.use_smem) {
    // Merge into the global table: the occupied slots are listed first (a
    // block scan), so each thread merges about one group, and every group's
    // global insert and atomics run in the same round instead of one after
    // another on the threads that hold several.
    __syncthreads();
    int c = 0;
    for (int i = threadIdx.x; i < p.sm_slots; i += kGroupThreads) c += s_keys[i] != kEmptySlot ? 1 : 0;
    int occupied;
    int o = block_exclusive_sum<kGroupThreads>(c, &occupied, s_scan);
    for (int i = threadIdx.x; i < p.sm_slots; i += kGroupThreads)
      if (s_keys[i] != kEmptySlot) s_occ[o++] = static_cast<uint16_t>(i);
    __syncthreads();
    for (int j = threadIdx.x; j < occupied; j += kGroupThreads) {
      const int i = s_occ[j];
      const uint64_t g = global_slot(p, s_keys[i], &s_claims);
      if (g == UINT64_MAX) continue;
      for (int a = 0; a < p.n_acc; ++a) acc_combine(p.accs + g * p.n_acc + a, p.acc[a].fn, p.acc[a].vt, s_acc[i * p.n_acc + a]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_claims != 0)
    atomicAdd(reinterpret_cast<unsigned long long*>(&p.st->aux[0]), s_claims);
}

// HyperLogLog sketch (Flajolet, Fusy, Gandouet, Meunier 2007) of a batch's
// packed keys: 2^12 registers, each the largest leading-zero rank + 1 of
// the hashes that fall in it. Registers gather per CTA in shared memory.
constexpr int kSketchBits = 12;
constexpr int kSketchRegs = 1 << kSketchBits;

__global__ void __launch_bounds__(256) group_sketch_kernel(const __grid_constant__ GroupParams p,
                                                           unsigned* __restrict__ regs) {
  __shared__ unsigned s_regs[kSketchRegs];
  for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x) s_regs[i] = 0;
  __syncthreads();
  const int64_t n = clamp_rows(p.n_dev, p.n_rows);
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    // a hash unrelated to the slot hash (another constant before the mixer)
    const uint64_t h = mix64(pack_key(p, r) ^ 0xd6e8feb86659fd93ull);
    const unsigned idx = static_cast<unsigned>(h >> (64 - kSketchBits));
    const unsigned rank = static_cast<unsigned>(__clzll((h << kSketchBits) | (1ull << (kSketchBits - 1)))) + 1u;
    if (rank > s_regs[idx]) atomicMax(&s_regs[idx], rank);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x) {
    const unsigned v = s_regs[i];
    if (v > *reinterpret_cast<volatile unsigned*>(regs + i)) atomicMax(regs + i, v);
  }
}

struct AccKinds {
  int8_t fn[kMaxAggs];
  int8_t vt[kMaxAggs];
};

__global__ void group_init_kernel(uint64_t* keys, unsigned long long* accs, uint64_t n_slots, int n_acc,
                                  AccKinds kinds) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n_slots; i += stride) {
    keys[i] = kEmptySlot;
    for (int a = 0; a < n_acc; ++a) accs[i * n_acc + a] = acc_init(kinds.fn[a], kinds.vt[a]);
  }
}

// Move every group of an old table into a larger one (accumulators copied).
__global__ void group_rehash_kernel(const uint64_t* old_keys, const unsigned long long* old_accs, uint64_t old_cap,
                                    uint64_t* keys, unsigned long long* accs, uint64_t mask, int n_acc, DevStatus* st) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i <= old_cap; i += stride) {
    const uint64_t key = old_keys[i];
    uint64_t dst;
    if (i == old_cap) {
      dst = mask + 1;  // special slot stays special
      if (key == kEmptySlot) {
        // the special slot's key word is never written; copy its accumulators
      }
    } else {
      if (key == kEmptySlot) continue;
      uint64_t slot = hash_key(static_cast<int64_t>(key)) & mask;
      bool ok = false;
      for (uint64_t k = 0; k <= mask; ++k) {
        const unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long*>(keys + slot),
                                                  static_cast<unsigned long long>(kEmptySlot),
                                                  static_cast<unsigned long long>(key));
        if (prev == kEmptySlot) {
          ok = true;
          break;
        }
        slot = (slot + 1) & mask;
      }
      if (!ok) {
        raise_status(st, GFPDB_ENOMEM, 21);
        continue;
      }
      dst = slot;
    }
    for (int a = 0; a < n_acc; ++a) accs[dst * n_acc + a] = old_accs[i * n_acc + a];
  }
}

struct OutAggDev {
  int8_t kind;  // 0: copy accumulator, 1: avg = sum / count
  int8_t out_type;  // DType code of the output column
  int8_t vt;
  int8_t pad;
  int32_t a0, a1;  // accumulator indices
  void* dst;
};

struct FinalParams {
  const uint64_t* keys;
  const unsigned long long* accs;
  uint64_t cap;  // special slot at index cap
  const int64_t* special_dev;  // non-zero once the all-ones key has a group
  int32_t n_acc;
  int32_t n_keys;
  int32_t n_out;
  int32_t key_bits[2];
  void* key_dst[2];
  int32_t key_type[2];
  OutAggDev outs[kMaxAggs];
  unsigned long long* counter;
};

__device__ __forceinline__ void store_typed(void* dst, int64_t pos, int type, int64_t v) {
  if (type == CT_I64 || type == CT_F64) static_cast<long long*>(dst)[pos] = v;
  else static_cast<int*>(dst)[pos] = static_cast<int32_t>(v);
}

// Each warp lists the live slots of kSteps consecutive 32-slot steps with
// one atomic on the output counter. Large tables take several steps per
// atomic (one address taking an atomic per 32 slots would queue them);
// small ones one step per warp, so that more warps share the few slots.
constexpr uint64_t kFinalChunkedSlots = 1ull << 20;

template <int kSteps>
__global__ void __launch_bounds__(256) group_finalize_kernel(const __grid_constant__ FinalParams p) {
  const int lane = threadIdx.x & 31;
  const uint32_t below = (1u << lane) - 1u;
  const uint64_t n_slots = p.cap + 1;
  const uint64_t warp0 = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  constexpr uint64_t kChunk = 32 * kSteps;
  for (uint64_t base = warp0 * kChunk; base < n_slots; base += n_warps * kChunk) {
    uint64_t key[kSteps];
    uint32_t m[kSteps];
    int total = 0;
#pragma unroll
    for (int k = 0; k < kSteps; ++k) {
      const uint64_t i = base + k * 32 + lane;
      bool live = false;
      key[k] = 0;
      if (i < p.cap) {
        key[k] = p.keys[i];
        live = key[k] != kEmptySlot;
      } else if (i == p.cap) {
        key[k] = kEmptySlot;
        live = *p.special_dev != 0;
      }
      m[k] = __ballot_sync(0xffffffffu, live);
      total += __popc(m[k]);
    }
    if (total == 0) continue;
    unsigned long long at = 0;
    if (lane == 0) at = atomicAdd(p.counter, static_cast<unsigned long long>(total));
    at = __shfl_sync(0xffffffffu, at, 0);
#pragma unroll
    for (int k = 0; k < kSteps; ++k) {
      if (m[k] >> lane & 1u) {
        const uint64_t i = base + k * 32 + lane;
        const int64_t pos = static_cast<int64_t>(at) + __popc(m[k] & below);
        if (p.n_keys == 1) {
          const int64_t v = p.key_bits[0] == 64 ? static_cast<int64_t>(key[k])
                                                : static_cast<int32_t>(static_cast<uint32_t>(key[k]));
          store_typed(p.key_dst[0], pos, p.key_type[0], v);
        } else if (p.n_keys == 2) {
          store_typed(p.key_dst[0], pos, p.key_type[0], static_cast<int32_t>(static_cast<uint32_t>(key[k] >> 32)));
          store_typed(p.key_dst[1], pos, p.key_type[1], static_cast<int32_t>(static_cast<uint32_t>(key[k])));
        }
        for (int j = 0; j < p.n_out; ++j) {
          const OutAggDev& o = p.outs[j];
          const unsigned long long a = p.accs[i * p.n_acc + o.a0];
          if (o.kind == 0) {
            store_typed(o.dst, pos, o.out_type, static_cast<int64_t>(a));
          } else {
            const unsigned long long c = p.accs[i * p.n_acc + o.a1];
            const double s = o.vt == VT_F64 ? __longlong_as_double(static_cast<long long>(a))
                                            : static_cast<double>(static_cast<long long>(a));
            const double avg = c == 0 ? 0.0 : s / static_cast<double>(c);
            static_cast<double*>(o.dst)[pos] = avg;
          }
        }
      }
      at += __popc(m[k]);
    }
  }
}

// ------------------------------------------------------- string dictionary

struct DictDev {
  uint64_t* slot_hash;
  uint32_t* slot_code;  // 0 = not published yet, else code + 1
  int64_t* code_off;
  int32_t* code_len;
  uint8_t* heap;
  uint64_t mask;
  int64_t code_cap;
  int64_t heap_cap;
  DevStatus* st;  // aux[0]: codes, aux[1]: heap bytes
};

__device__ __forceinline__ uint64_t dict_hash(const uint8_t* s, int32_t n) {
  uint64_t h = hash_bytes(s, n);
  return h == kEmptySlot ? kEmptySlot - 1 : h;
}

// Values are utf8 strings (offs, bytes) or, with offs null, fixed-width
// records of `width` bytes each.
__global__ void __launch_bounds__(256) dict_encode_kernel(const int32_t* __restrict__ offs, const uint8_t* __restrict__ bytes,
                                                          int32_t width, int64_t n, int32_t* __restrict__ out_codes,
                                                          DictDev d) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const int64_t b = offs != nullptr ? offs[r] : r * width;
    const int32_t len = offs != nullptr ? offs[r + 1] - static_cast<int32_t>(b) : width;
    const uint8_t* str = bytes + b;
    const uint64_t h = dict_hash(str, len);
    uint64_t slot = h & d.mask;
    int32_t code = -1;
    for (uint64_t i = 0; i <= d.mask && code < 0; ++i, slot = (slot + 1) & d.mask) {
      uint64_t s = *reinterpret_cast<volatile uint64_t*>(d.slot_hash + slot);
      if (s == kEmptySlot) {
        s = atomicCAS(reinterpret_cast<unsigned long long*>(d.slot_hash + slot),
                      static_cast<unsigned long long>(kEmptySlot), static_cast<unsigned long long>(h));
        if (s == kEmptySlot) {
          // This thread owns the new entry: store its bytes, then publish.
          const unsigned long long c = atomicAdd(reinterpret_cast<unsigned long long*>(&d.st->aux[0]), 1ull);
          const unsigned long long off = atomicAdd(reinterpret_cast<unsigned long long*>(&d.st->aux[1]),
                                                   static_cast<unsigned long long>(len));
          if (static_cast<int64_t>(c) >= d.code_cap || static_cast<int64_t>(off) + len > d.heap_cap) {
            raise_status(d.st, GFPDB_ENOMEM, 30);
            st_release32(d.slot_code + slot, 0xFFFFFFFFu);
            break;
          }
          for (int32_t k = 0; k < len; ++k) d.heap[off + k] = str[k];
          d.code_off[c] = static_cast<int64_t>(off);
          d.code_len[c] = len;
          __threadfence();
          st_release32(d.slot_code + slot, static_cast<uint32_t>(c) + 1u);
          code = static_cast<int32_t>(c);
          break;
        }
      }
      if (s != h) continue;
      // Same hash: wait (bounded) until the owner has published, then compare bytes.
      uint32_t pub = 0;
      for (uint32_t spin = 0; spin < kDictSpinLimit; ++spin) {
        pub = ld_acquire32(d.slot_code + slot);
        if (pub != 0) break;
        __nanosleep(32);
      }
      if (pub == 0) {
        raise_status(d.st, GFPDB_ETIMEDOUT, 31);
        break;
      }
      if (pub == 0xFFFFFFFFu) break;  // owner ran out of space; error already raised
      const int32_t c = static_cast<int32_t>(pub - 1u);
      if (d.code_len[c] != len) continue;
      const uint8_t* other = d.heap + d.code_off[c];
      bool eq = true;
      for (int32_t k = 0; eq && k < len; ++k) eq = other[k] == str[k];
      if (eq) code = c;
    }
    if (code < 0) raise_status(d.st, GFPDB_ENOMEM, 32);
    out_codes[r] = code < 0 ? 0 : code;
  }
}

__global__ void dict_rehash_kernel(DictDev d, int64_t n_codes) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; c < n_codes; c += stride) {
    const uint64_t h = dict_hash(d.heap + d.code_off[c], d.code_len[c]);
    uint64_t slot = h & d.mask;
    for (uint64_t i = 0; i <= d.mask; ++i, slot = (slot + 1) & d.mask) {
      const unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long*>(d.slot_hash + slot),
                                                static_cast<unsigned long long>(kEmptySlot),
                                                static_cast<unsigned long long>(h));
      if (prev == kEmptySlot) {
        d.slot_code[slot] = static_cast<uint32_t>(c) + 1u;
        break;
      }
    }
  }
}

__global__ void dict_lengths_kernel(const int32_t* codes, int64_t n, const int32_t* code_len, int32_t* lens) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride)
    lens[r] = code_len[codes[r]];
}

// Key records: each record's values written at fixed offsets (4-byte words;
// an 8-byte value as two), and back into columns.
struct RecordCols {
  DevCol cols[kMaxKeyColumns];
  int32_t off[kMaxKeyColumns];    // byte offset of the column in a record
  int32_t width[kMaxKeyColumns];  // 4 or 8
  int32_t n_cols;
  int32_t rec_width;              // multiple of 4
};

__global__ void group_record_pack_kernel(const __grid_constant__ RecordCols rc, int64_t n, uint32_t* out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int words = rc.rec_width / 4;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    uint32_t* rec = out + r * words;
    for (int k = 0; k < rc.n_cols; ++k) {
      const int64_t v = load_int(rc.cols[k], r);
      rec[rc.off[k] / 4] = static_cast<uint32_t>(v);
      if (rc.width[k] == 8) rec[rc.off[k] / 4 + 1] = static_cast<uint32_t>(static_cast<uint64_t>(v) >> 32);
    }
  }
}

__global__ void group_record_split_kernel(const __grid_constant__ RecordCols rc, int64_t n, const int32_t* codes,
                                          const int64_t* code_off, const uint8_t* heap, void* const* dst) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const uint32_t* rec = reinterpret_cast<const uint32_t*>(heap + code_off[codes[r]]);
    for (int k = 0; k < rc.n_cols; ++k) {
      const uint32_t lo = rec[rc.off[k] / 4];
      if (rc.width[k] == 8)
        static_cast<uint64_t*>(dst[k])[r] = (static_cast<uint64_t>(rec[rc.off[k] / 4 + 1]) << 32) | lo;
      else
        static_cast<uint32_t*>(dst[k])[r] = lo;
    }
  }
}

__global__ void dict_copy_kernel(const int32_t* codes, int64_t n, const int64_t* code_off, const uint8_t* heap,
                                 const int32_t* offs, uint8_t* out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const uint8_t* src = heap + code_off[codes[r]];
    const int32_t o = offs[r], len = offs[r + 1] - o;
    for (int32_t k = 0; k < len; ++k) out[o + k] = src[k];
  }
}

int grid_for(int64_t n) {
  int64_t blocks = (n + 255) / 256;
  int64_t cap = static_cast<int64_t>(num_sms()) * 8;
  if (blocks > cap) blocks = cap;
  return static_cast<int>(blocks < 1 ? 1 : blocks);
}

// Tables above this many slots (32 MB of keys) are sized by a sketch when
// the batch allows it.
constexpr uint64_t kSketchMinSlots = 1ull << 22;

bool stream_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus c = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &c) == cudaSuccess && c != cudaStreamCaptureStatusNone;
}

uint64_t next_pow2(uint64_t x) {
  uint64_t c = 1;
  while (c < x) c <<= 1;
  return c;
}

DevStatus read_status(const DevStatus* d, cudaStream_t s) {
  DevStatus h;
  GF_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  sync(s);
  return h;
}

// Distinct keys of a batch, estimated from its HyperLogLog sketch (the raw
// estimate alpha_m m^2 / sum 2^-M[j], with linear counting over the empty
// registers in the small range); standard error about 1.04 / sqrt(2^12).
double sketch_distinct(const GroupParams& p, int64_t n, cudaStream_t s) {
  auto regs = make_filled(kSketchRegs * 4, 0, s);
  // enough CTAs to stream the keys at full occupancy (16 KB of registers
  // each); their merges mostly find the global registers already as large
  int64_t blocks = (n + 1023) / 1024;
  if (blocks > static_cast<int64_t>(num_sms()) * 8) blocks = static_cast<int64_t>(num_sms()) * 8;
  {
    ProfScope prof("group_sketch_kernel", s);
    group_sketch_kernel<<<static_cast<int>(blocks < 1 ? 1 : blocks), 256, 0, s>>>(p, regs->as<unsigned>());
    after_launch("group_sketch_kernel");
    prof.stop(static_cast<double>(n) * 8);
  }
  std::vector<unsigned> h(kSketchRegs);
  GF_CUDA(cudaMemcpyAsync(h.data(), regs->data(), kSketchRegs * 4, cudaMemcpyDeviceToHost, s));
  sync(s);
  double sum = 0;
  int zeros = 0;
  for (unsigned v : h) {
    sum += std::ldexp(1.0, -static_cast<int>(v));
    zeros += v == 0 ? 1 : 0;
  }
  const double m = kSketchRegs;
  double e = 0.7213 / (1.0 + 1.079 / m) * m * m / sum;
  if (e <= 2.5 * m && zeros > 0) e = m * std::log(m / zeros);
  return e;
}

class StringDict {
 public:
  BufferPtr slot_hash, slot_code, code_off, code_len, heap, status;
  uint64_t cap = 0;
  int64_t code_cap = 0, heap_cap = 0;
  int64_t codes_upper = 0, heap_upper = 0;  // host-side upper bounds

  DictDev dev() const {
    DictDev d;
    d.slot_hash = slot_hash->as<uint64_t>();
    d.slot_code = slot_code->as<uint32_t>();
    d.code_off = code_off->as<int64_t>();
    d.code_len = code_len->as<int32_t>();
    d.heap = heap->as<uint8_t>();
    d.mask = cap - 1;
    d.code_cap = code_cap;
    d.heap_cap = heap_cap;
    d.st = status->as<DevStatus>();
    return d;
  }

  void ensure(int64_t more_codes, int64_t more_bytes, cudaStream_t s) {
    if (!status) status = make_filled(sizeof(DevStatus), 0, s);
    int64_t codes_real = 0, bytes_real = 0;
    const bool grow_slots = static_cast<uint64_t>(2 * (codes_upper + more_codes)) > cap;
    const bool grow_codes = codes_upper + more_codes > code_cap;
    const bool grow_heap = heap_upper + more_bytes > heap_cap;
    if (!(grow_slots || grow_codes || grow_heap)) return;
    if (cap > 0) {
      DevStatus h = read_status(status->as<DevStatus>(), s);
      raise_device_status(h, "string dictionary");
      codes_real = h.aux[0];
      bytes_real = h.aux[1];
      codes_upper = codes_real;
      heap_upper = bytes_real;
    }
    const int64_t need_codes = codes_upper + more_codes;
    const int64_t need_bytes = heap_upper + more_bytes;
    if (need_codes > code_cap) {
      int64_t nc = static_cast<int64_t>(next_pow2(static_cast<uint64_t>(need_codes < 1024 ? 1024 : need_codes)));
      auto off = make_buffer(nc * 8, s), len = make_buffer(nc * 4, s);
      if (codes_real > 0) {
        GF_CUDA(cudaMemcpyAsync(off->data(), code_off->data(), codes_real * 8, cudaMemcpyDeviceToDevice, s));
        GF_CUDA(cudaMemcpyAsync(len->data(), code_len->data(), codes_real * 4, cudaMemcpyDeviceToDevice, s));
      }
      code_off = off;
      code_len = len;
      code_cap = nc;
    }
    if (need_bytes > heap_cap) {
      int64_t nb = static_cast<int64_t>(next_pow2(static_cast<uint64_t>(need_bytes < 4096 ? 4096 : need_bytes)));
      auto hp = make_buffer(nb, s);
      if (bytes_real > 0) GF_CUDA(cudaMemcpyAsync(hp->data(), heap->data(), bytes_real, cudaMemcpyDeviceToDevice, s));
      heap = hp;
      heap_cap = nb;
    }
    uint64_t want = next_pow2(static_cast<uint64_t>(2 * need_codes < 1024 ? 1024 : 2 * need_codes));
    if (want > cap) {
      slot_hash = make_filled(static_cast<int64_t>(want) * 8, 0xFF, s);
      slot_code = make_filled(static_cast<int64_t>(want) * 4, 0, s);
      cap = want;
      if (codes_real > 0) {
        dict_rehash_kernel<<<grid_for(codes_real), 256, 0, s>>>(dev(), codes_real);
        after_launch("dict_rehash_kernel");
      }
    }
  }

  BufferPtr encode(const Column& c, cudaStream_t s) {
    const int64_t n = c.length;
    int32_t ends[2] = {0, 0};
    if (n > 0) {
      GF_CUDA(cudaMemcpyAsync(&ends[0], c.offsets, 4, cudaMemcpyDeviceToHost, s));
      GF_CUDA(cudaMemcpyAsync(&ends[1], c.offsets + n, 4, cudaMemcpyDeviceToHost, s));
      sync(s);
    }
    ensure(n, ends[1] - ends[0], s);
    auto codes = make_buffer(n * 4, s);
    if (n > 0) {
      dict_encode_kernel<<<grid_for(n), 256, 0, s>>>(c.offsets, static_cast<const uint8_t*>(c.data), 0, n,
                                                     codes->as<int32_t>(), dev());
      after_launch("dict_encode_kernel");
    }
    codes_upper += n;
    heap_upper += ends[1] - ends[0];
    return codes;
  }

  // n records of `width` bytes each (4-byte aligned; the heap keeps every
  // record at a multiple of its width, so records stay aligned).
  BufferPtr encode_records(const void* records, int64_t n, int32_t width, cudaStream_t s) {
    ensure(n, n * width, s);
    auto codes = make_buffer(n * 4, s);
    if (n > 0) {
      dict_encode_kernel<<<grid_for(n), 256, 0, s>>>(nullptr, static_cast<const uint8_t*>(records), width, n,
                                                     codes->as<int32_t>(), dev());
      after_launch("dict_encode_kernel");
    }
    codes_upper += n;
    heap_upper += n * width;
    return codes;
  }

  ColumnPtr decode(const int32_t* codes, int64_t n, cudaStream_t s) {
    auto offs = make_buffer((n + 1) * 4, s);
    int64_t total = 0;
    if (n > 0) {
      auto lens = make_buffer(n * 4, s);
      dict_lengths_kernel<<<grid_for(n), 256, 0, s>>>(codes, n, code_len->as<int32_t>(), lens->as<int32_t>());
      after_launch("dict_lengths_kernel");
      total = exclusive_scan_i32(lens->as<int32_t>(), offs->as<int32_t>(), n, s);
    } else {
      GF_CUDA(cudaMemsetAsync(offs->data(), 0, 4, s));
    }
    auto bytes = make_buffer(total, s);
    if (n > 0 && total > 0) {
      dict_copy_kernel<<<grid_for(n), 256, 0, s>>>(codes, n, code_off->as<int64_t>(), heap->as<uint8_t>(),
                                                   offs->as<int32_t>(), bytes->as<uint8_t>());
      after_launch("dict_copy_kernel");
    }
    return make_utf8_column(n, offs, bytes);
  }
};

}  // namespace

class GroupTable {
 public:
  std::vector<std::string> group_cols;
  std::vector<GroupAggregate> aggs;
  int64_t hint = 0;

  bool compiled = false;
  std::vector<DType> key_types;
  std::vector<int32_t> key_bits;
  std::vector<AccDev> accs;           // internal accumulators
  std::vector<OutAggDev> outs;        // user aggregates -> accumulators
  std::vector<DType> out_types;
  Program prog{};
  ColumnSlots slots;
  std::vector<std::unique_ptr<StringDict>> dicts;  // per key column (utf8 only)
  bool wide = false;                        // keys as records, grouped by record code
  RecordCols records{};
  std::unique_ptr<StringDict> record_dict;

  BufferPtr keys, accbuf, status, fnvt;
  uint64_t cap = 0;
  int64_t groups_upper = 0;

  void compile(const TupleSet& ts) {
    if (group_cols.size() > static_cast<size_t>(kMaxKeyColumns))
      fail(GFPDB_EUNSUPPORTED, "group-by over more than 8 key columns");
    int bits = 0;
    for (auto& g : group_cols) {
      DType t = ts.field(ts.require_column(g)).type;
      if (t == DType::Float64) fail(GFPDB_EUNSUPPORTED, "float64 group keys");
      key_types.push_back(t);
      int b = t == DType::Int64 ? 64 : 32;
      key_bits.push_back(b);
      bits += b;
      dicts.emplace_back(t == DType::Utf8 ? new StringDict() : nullptr);
    }
    if (group_cols.size() > 2 || bits > 64) {
      wide = true;
      std::memset(&records, 0, sizeof(records));
      records.n_cols = static_cast<int32_t>(group_cols.size());
      for (size_t k = 0; k < group_cols.size(); ++k) {
        records.off[k] = records.rec_width;
        records.width[k] = key_types[k] == DType::Int64 ? 8 : 4;  // utf8 columns as their int32 codes
        records.rec_width += records.width[k];
      }
      record_dict.reset(new StringDict());
    }
    std::memset(&prog, 0, sizeof(prog));
    for (auto& a : aggs) {
      OutAggDev o{};
      auto add_acc = [&](int8_t fn, int8_t vt, Operand in) {
        if (static_cast<int>(accs.size()) >= kMaxAggs) fail(GFPDB_EUNSUPPORTED, "too many aggregates");
        AccDev d{};
        d.fn = fn;
        d.vt = vt;
        d.in = in;
        accs.push_back(d);
        return static_cast<int32_t>(accs.size() - 1);
      };
      if (a.fn == AGG_AVG_REDUCE) {
        // AvgReduce (fpdb-executor/src/physical/aggregate/function/AvgReduce.cpp:21-84):
        // the first phase's AVG_INTERMEDIATE_SUM_<name> and
        // AVG_INTERMEDIATE_COUNT_<name> columns, each summed, divided at
        // finalisation.
        auto column = [](const std::string& n) {
          auto e = std::make_shared<Expr>();
          e->kind = Expr::Column;
          e->name = n;
          return ExprPtr(e);
        };
        DType sum_t, cnt_t;
        Operand sum_in = compile_value(column(kAvgIntermediateSum + a.name), ts.fields(), prog, slots, &sum_t);
        Operand cnt_in = compile_value(column(kAvgIntermediateCount + a.name), ts.fields(), prog, slots, &cnt_t);
        if (cnt_t == DType::Float64 || cnt_t == DType::Utf8 || sum_t == DType::Utf8)
          fail(GFPDB_EINVAL, "AVG_REDUCE '" + a.name + "' needs a numeric sum and an integer count column");
        o.kind = 1;
        o.vt = sum_t == DType::Float64 ? VT_F64 : VT_I64;
        o.a0 = add_acc(AGG_SUM, o.vt, sum_in);
        o.a1 = add_acc(AGG_SUM, VT_I64, cnt_in);
        o.out_type = static_cast<int8_t>(DType::Float64);
        out_types.push_back(DType::Float64);
      } else if (a.fn == AGG_COUNT_STAR || (a.fn == AGG_COUNT && !a.expr)) {
        Operand none{};
        none.kind = OPND_LIT;
        o.kind = 0;
        o.a0 = add_acc(AGG_COUNT_STAR, VT_I64, none);
        o.out_type = static_cast<int8_t>(DType::Int64);
        out_types.push_back(DType::Int64);
      } else {
        if (!a.expr) fail(GFPDB_EINVAL, "aggregate '" + a.name + "' needs an input expression");
        DType in_t;
        Operand in = compile_value(a.expr, ts.fields(), prog, slots, &in_t);
        const int8_t vt = in_t == DType::Float64 ? VT_F64 : VT_I64;
        if (a.fn == AGG_SUM) {
          o.a0 = add_acc(AGG_SUM, vt, in);
          DType ot = vt == VT_F64 ? DType::Float64 : DType::Int64;
          o.out_type = static_cast<int8_t>(ot);
          out_types.push_back(ot);
        } else if (a.fn == AGG_COUNT) {
          o.a0 = add_acc(AGG_COUNT, VT_I64, in);
          o.out_type = static_cast<int8_t>(DType::Int64);
          out_types.push_back(DType::Int64);
        } else if (a.fn == AGG_MIN || a.fn == AGG_MAX) {
          o.a0 = add_acc(a.fn, vt, in);
          o.out_type = static_cast<int8_t>(in_t);
          out_types.push_back(in_t);
        } else {  // AVG: sum and count, divided at finalisation
          o.kind = 1;
          o.vt = vt;
          o.a0 = add_acc(AGG_SUM, vt, in);
          Operand none{};
          none.kind = OPND_LIT;
          o.a1 = add_acc(AGG_COUNT_STAR, VT_I64, none);
          o.out_type = static_cast<int8_t>(DType::Float64);
          out_types.push_back(DType::Float64);
        }
      }
      outs.push_back(o);
    }
    compiled = true;
  }

  void init_table(uint64_t new_cap, cudaStream_t s) {
    const int na = static_cast<int>(accs.size());
    // Empty keys are all-ones and sum / count accumulators start at zero, so
    // without MIN / MAX the table comes pre-filled (no init kernel; inside a
    // captured plan from the graph's fill regions).
    bool zero_init = true;
    for (int a = 0; a < na; ++a) zero_init &= accs[a].fn != AGG_MIN && accs[a].fn != AGG_MAX;
    const int64_t key_bytes = static_cast<int64_t>(new_cap + 1) * 8;
    const int64_t acc_bytes = static_cast<int64_t>(new_cap + 1) * 8 * (na > 0 ? na : 1);
    BufferPtr nk, na_buf;
    if (zero_init) {
      nk = make_filled(key_bytes, 0xFF, s);
      na_buf = make_filled(acc_bytes, 0, s);
    } else {
      nk = make_buffer(key_bytes, s);
      na_buf = make_buffer(acc_bytes, s);
      AccKinds kinds{};
      for (int a = 0; a < na; ++a) {
        kinds.fn[a] = accs[a].fn;
        kinds.vt[a] = accs[a].vt;
      }
      group_init_kernel<<<grid_for(static_cast<int64_t>(new_cap + 1)), 256, 0, s>>>(
          nk->as<uint64_t>(), na_buf->as<unsigned long long>(), new_cap + 1, na, kinds);
      after_launch("group_init_kernel");
    }
    if (!status) status = make_filled(sizeof(DevStatus), 0, s);
    if (cap > 0) {
      group_rehash_kernel<<<grid_for(static_cast<int64_t>(cap + 1)), 256, 0, s>>>(
          keys->as<uint64_t>(), accbuf->as<unsigned long long>(), cap, nk->as<uint64_t>(),
          na_buf->as<unsigned long long>(), new_cap - 1, na, status->as<DevStatus>());
      after_launch("group_rehash_kernel");
    }
    keys = nk;
    accbuf = na_buf;
    cap = new_cap;
  }

  void update(const TupleSet& batch, cudaStream_t s) {
    if (!compiled) compile(batch);
    // String keys are dictionary-encoded from exact inputs; other batches
    // may carry their row count on the device.
    TupleSetPtr exact_holder;
    const TupleSet* tsp = &batch;
    bool utf8_key = false;
    for (auto t : key_types) utf8_key |= t == DType::Utf8;
    if ((utf8_key || wide) && !batch.exact()) {
      exact_holder = batch.resolve(s);
      tsp = exact_holder.get();
    }
    const TupleSet& ts = *tsp;
    const int64_t n = ts.num_rows();
    if (n >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "group-by batch must have fewer than 2^31 rows");

    GroupParams* pp = new GroupParams;
    std::unique_ptr<GroupParams> holder(pp);
    GroupParams& p = *pp;
    std::memset(&p, 0, sizeof(p));
    p.n_rows = n;
    p.n_dev = ts.rows_dev();
    p.n_keys = static_cast<int32_t>(group_cols.size());
    p.n_acc = static_cast<int32_t>(accs.size());
    std::vector<BufferPtr> code_bufs;
    if (wide && n > 0) {
      RecordCols rc = records;
      for (int k = 0; k < rc.n_cols; ++k) {
        const auto& c = ts.column(group_cols[k]);
        if (c->type != key_types[k]) fail(GFPDB_EINVAL, "group key column changed type between batches");
        if (c->type == DType::Utf8) {
          auto codes = dicts[k]->encode(*c, s);
          code_bufs.push_back(codes);
          rc.cols[k] = DevCol{codes->data(), nullptr, CT_I32, 0};
        } else {
          rc.cols[k] = DevCol{c->data, nullptr, static_cast<int32_t>(c->type), 0};
        }
      }
      auto recs = make_buffer(n * rc.rec_width, s);
      group_record_pack_kernel<<<grid_for(n), 256, 0, s>>>(rc, n, recs->as<uint32_t>());
      after_launch("group_record_pack_kernel");
      auto codes = record_dict->encode_records(recs->data(), n, rc.rec_width, s);
      code_bufs.push_back(codes);
      p.n_keys = 1;
      p.key_bits[0] = 32;
      p.key_cols[0] = DevCol{codes->data(), nullptr, CT_I32, 0};
    } else if (n > 0) {
      for (int k = 0; k < p.n_keys; ++k) {
        const auto& c = ts.column(group_cols[k]);
        if (c->type != key_types[k]) fail(GFPDB_EINVAL, "group key column changed type between batches");
        p.key_bits[k] = key_bits[k];
        if (c->type == DType::Utf8) {
          auto codes = dicts[k]->encode(*c, s);
          code_bufs.push_back(codes);
          p.key_cols[k] = DevCol{codes->data(), nullptr, CT_I32, 0};
        } else {
          p.key_cols[k] = DevCol{c->data, nullptr, static_cast<int32_t>(c->type), 0};
        }
      }
    }

    // Size the table so that it stays at most half full.
    int64_t bound = groups_upper + n;
    if (hint > 0 && bound > hint) bound = groups_upper > hint ? groups_upper : hint;
    uint64_t want = next_pow2(static_cast<uint64_t>(2 * bound < 1024 ? 1024 : 2 * bound));
    if (want > cap && cap > 0) {
      // Upper bound says grow: read the real group count first.
      DevStatus h = read_status(status->as<DevStatus>(), s);
      raise_device_status(h, "group-by");
      groups_upper = h.aux[0];
      bound = groups_upper + n;
      if (hint > 0 && bound > hint) bound = groups_upper > hint ? groups_upper : hint;
      want = next_pow2(static_cast<uint64_t>(2 * bound < 1024 ? 1024 : 2 * bound));
    }
    if (want > cap && want > kSketchMinSlots && hint == 0 && n > 0 && p.n_keys > 0 && ts.exact() &&
        !deferred_mode() && !stream_capturing(s)) {
      // A large table for a batch whose rows are on the host: size it for
      // the batch's estimated distinct keys (with a quarter to spare) over
      // the exact groups so far instead of its row count.
      const double est = sketch_distinct(p, n, s);
      int64_t fresh = static_cast<int64_t>(est * 1.25) + 1024;
      if (fresh > n) fresh = n;
      const int64_t known = cap > 0 ? groups_upper : 0;  // exact: read above
      const int64_t b2 = known + fresh;
      const uint64_t w2 = next_pow2(static_cast<uint64_t>(2 * b2 < 1024 ? 1024 : 2 * b2));
      if (w2 < want) want = w2 > cap ? w2 : cap;
    }
    if (want > cap) init_table(want, s);
    if (n == 0) return;

    for (int a = 0; a < p.n_acc; ++a) p.acc[a] = accs[a];
    bind_columns(slots, ts, p.cols, kMaxCols);
    p.prog = prog;
    p.keys = keys->as<uint64_t>();
    p.accs = accbuf->as<unsigned long long>();
    p.mask = cap - 1;
    p.st = status->as<DevStatus>();
    // Shared-memory pre-aggregation unless the caller expects many groups.
    const int per_slot = 8 + 8 * p.n_acc;
    int sm_slots = kGroupSmemSlotsMax;
    // dynamic plus static shared memory stays within the 48 KB a launch
    // gets without opting in to more
    while (sm_slots * per_slot > 44 * 1024) sm_slots >>= 1;
    p.use_smem = (hint == 0 || hint <= 4096) ? 1 : 0;
    p.sm_slots = sm_slots;
    const size_t dyn = p.use_smem ? static_cast<size_t>(sm_slots) * per_slot : 0;
    int64_t blocks = (n + kGroupThreads * 16 - 1) / (kGroupThreads * 16);
    // one wave: as many CTAs as fit on every SM at once
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, group_update_kernel, kGroupThreads, dyn) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    int64_t max_blocks = static_cast<int64_t>(num_sms()) * per_sm;
    if (blocks > max_blocks) blocks = max_blocks;
    if (blocks < 1) blocks = 1;
    ProfScope prof("group_update_kernel", s);
    group_update_kernel<<<static_cast<int>(blocks), kGroupThreads, dyn, s>>>(p);
    after_launch("group_update_kernel");
    double w = 0;
    for (int k = 0; k < p.n_keys; ++k) w += p.key_bits[k] / 8;
    if (wide) w += records.rec_width - 4;
    for (size_t i = 0; i < slots.types.size(); ++i) w += dtype_width(slots.types[i]);
    prof.stop(static_cast<double>(n) * w);
    if (p.n_dev) prof.set_bytes_model(p.n_dev, n, w, nullptr, 0, ts.rows_owner());
    groups_upper += n;
    if (hint > 0 && groups_upper > hint) groups_upper = hint;
  }

  TupleSetPtr finalize(const TupleSet* schema_src, cudaStream_t s) {
    std::vector<Field> fields;
    for (size_t k = 0; k < group_cols.size(); ++k)
      fields.push_back(Field{group_cols[k], compiled ? key_types[k] : DType::Int64});
    for (size_t j = 0; j < aggs.size(); ++j)
      fields.push_back(Field{aggs[j].name, compiled ? out_types[j] : DType::Int64});
    if (!compiled || cap == 0) return TupleSet::make_empty(fields, s);
    (void)schema_src;
    bool utf8_key = wide;
    for (auto t : key_types) utf8_key |= t == DType::Utf8;
    // Deferred: outputs sized for every slot, the group count stays on the
    // device and the status block is checked at the end of the plan.
    const bool defer = deferred_mode() && !utf8_key;
    int64_t n_groups = static_cast<int64_t>(cap) + 1;
    if (defer) {
      defer_check(status, status->as<DevStatus>(), "group-by");
    } else {
      DevStatus h = read_status(status->as<DevStatus>(), s);
      raise_device_status(h, "group-by");
      for (auto& d : dicts)
        if (d && d->status) raise_device_status(read_status(d->status->as<DevStatus>(), s), "string dictionary");
      if (record_dict && record_dict->status)
        raise_device_status(read_status(record_dict->status->as<DevStatus>(), s), "group key dictionary");
      n_groups = h.aux[0];
    }
    FinalParams fp;
    std::memset(&fp, 0, sizeof(fp));
    fp.keys = keys->as<uint64_t>();
    fp.accs = accbuf->as<unsigned long long>();
    fp.cap = cap;
    fp.special_dev = &status->as<DevStatus>()->aux[1];
    fp.n_acc = static_cast<int32_t>(accs.size());
    fp.n_keys = static_cast<int32_t>(group_cols.size());
    std::vector<BufferPtr> key_out(group_cols.size());
    BufferPtr record_codes;
    if (wide) {  // the table's key is the record code
      fp.n_keys = 1;
      record_codes = make_buffer(n_groups * 4, s);
      fp.key_dst[0] = record_codes->data();
      fp.key_type[0] = CT_I32;
      fp.key_bits[0] = 32;
    }
    for (size_t k = 0; k < group_cols.size() && !wide; ++k) {
      DType t = key_types[k] == DType::Utf8 ? DType::Int32 : key_types[k];
      key_out[k] = make_buffer(n_groups * dtype_width(t), s);
      fp.key_dst[k] = key_out[k]->data();
      fp.key_type[k] = static_cast<int32_t>(t);
      fp.key_bits[k] = key_bits[k];
    }
    std::vector<BufferPtr> agg_out(aggs.size());
    fp.n_out = static_cast<int32_t>(aggs.size());
    for (size_t j = 0; j < aggs.size(); ++j) {
      agg_out[j] = make_buffer(n_groups * dtype_width(out_types[j]), s);
      fp.outs[j] = outs[j];
      fp.outs[j].dst = agg_out[j]->data();
    }
    auto counter = make_filled(8, 0, s);
    fp.counter = counter->as<unsigned long long>();
    {
      ProfScope prof("group_finalize_kernel", s);
      if (cap + 1 >= kFinalChunkedSlots)
        group_finalize_kernel<8><<<grid_for(static_cast<int64_t>((cap + 1) / 8)), 256, 0, s>>>(fp);
      else
        group_finalize_kernel<1><<<grid_for(static_cast<int64_t>(cap + 1)), 256, 0, s>>>(fp);
      after_launch("group_finalize_kernel");
      prof.stop(static_cast<double>(cap + 1) * 8);
    }
    if (wide) {
      std::vector<void*> dst(group_cols.size());
      for (size_t k = 0; k < group_cols.size(); ++k) {
        key_out[k] = make_buffer(n_groups * records.width[k], s);
        dst[k] = key_out[k]->data();
      }
      auto dst_dev = make_buffer(static_cast<int64_t>(dst.size() * sizeof(void*)), s);
      GF_CUDA(cudaMemcpyAsync(dst_dev->data(), dst.data(), dst.size() * sizeof(void*), cudaMemcpyHostToDevice, s));
      if (n_groups > 0) {
        group_record_split_kernel<<<grid_for(n_groups), 256, 0, s>>>(
            records, n_groups, record_codes->as<int32_t>(), record_dict->code_off->as<int64_t>(),
            record_dict->heap->as<uint8_t>(), dst_dev->as<void*>());
        after_launch("group_record_split_kernel");
      }
      sync(s);  // dst (host vector) is read by the copy above
    }
    std::vector<ColumnPtr> cols;
    for (size_t k = 0; k < group_cols.size(); ++k) {
      if (key_types[k] == DType::Utf8) cols.push_back(dicts[k]->decode(key_out[k]->as<int32_t>(), n_groups, s));
      else cols.push_back(make_fixed_column(key_types[k], n_groups, key_out[k]));
    }
    for (size_t j = 0; j < aggs.size(); ++j) cols.push_back(make_fixed_column(out_types[j], n_groups, agg_out[j]));
    if (defer)
      return TupleSet::make_deferred(std::move(fields), std::move(cols), n_groups, counter,
                                     reinterpret_cast<const int64_t*>(counter->data()));
    return TupleSet::make(std::move(fields), std::move(cols), n_groups);
  }
};

std::shared_ptr<GroupTable> group_table_create(const std::vector<std::string>& group_cols,
                                               const std::vector<GroupAggregate>& aggs, int64_t groups_hint) {
  auto g = std::make_shared<GroupTable>();
  g->group_cols = group_cols;
  g->aggs = aggs;
  g->hint = groups_hint;
  return g;
}

void group_table_update(GroupTable& g, const TupleSet& batch, cudaStream_t s) { g.update(batch, s); }

TupleSetPtr group_table_finalize(GroupTable& g, cudaStream_t s) { return g.finalize(nullptr, s); }

}  // namespace gfpdb
